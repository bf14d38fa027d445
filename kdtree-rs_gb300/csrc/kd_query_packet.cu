// kd_query_packet.cu -- launches of the packet traversal (kd_query_packet.cuh)
// for the compile-time widths 2, 3, 8 and 16, the L1 / L2 / L-inf metrics and
// k <= 64 (k-best lists of 1, 4, 8, 16, 32 or 64 slots);
// a translation unit of its own so it compiles in parallel with the other
// query kernels.
#include <cstdlib>
#include <type_traits>

#include "kd_internal.hpp"

namespace kd {
namespace {

#include "kd_query_common.cuh"
#include "kd_lazy_best.cuh"
#include "kd_query_packet.cuh"

// The shared-memory share of the unified L1 / shared storage the packet
// kernels ask for (cudaFuncAttributePreferredSharedMemoryCarveout, percent):
// the heaps live in shared memory, the tree's nodes, boxes and rows come
// through L1.  With 16-slot heaps (26 KB per block) 90 % -- seven blocks per
// SM, the rest for L1 -- measured best on GB300 (N = 1M, d = 3, k = 16, 1M
// queries: 2.69 ms a step against 2.79 ms at 75 %, 2.99 ms at 60 % and
// 2.70 ms at 100 %).  KD_PACKET_CARVEOUT (0..100) overrides it for every k;
// unset, the other k keep the CUDA runtime's default.
int carveout_override() {
  static const int v = [] {
    const char* e = std::getenv("KD_PACKET_CARVEOUT");
    return e ? std::atoi(e) : -1;
  }();
  return v;
}

template <int K, typename F>
void apply_carveout(F* kernel) {
  int v = carveout_override();
  if (v < 0 && K == 16) v = 90;
  if (v >= 0) cudaFuncSetAttribute(kernel, cudaFuncAttributePreferredSharedMemoryCarveout, v);
}

template <int M, int D>
int launch_k(const QArgs& a, cudaStream_t st) {
  const unsigned blocks = static_cast<unsigned>((a.nq + QUERY_THREADS - 1) / QUERY_THREADS);
  if (a.k == 1) {
    apply_carveout<1>(k_query_packet<M, D, 1>);
    k_query_packet<M, D, 1><<<blocks, QUERY_THREADS, 0, st>>>(a);
  } else if (a.k <= 4) {
    apply_carveout<4>(k_query_packet<M, D, 4>);
    k_query_packet<M, D, 4><<<blocks, QUERY_THREADS, 0, st>>>(a);
  } else if (a.k <= 8) {
    apply_carveout<8>(k_query_packet<M, D, 8>);
    k_query_packet<M, D, 8><<<blocks, QUERY_THREADS, 0, st>>>(a);
  } else if (a.k <= 16) {
    apply_carveout<16>(k_query_packet<M, D, 16>);
    k_query_packet<M, D, 16><<<blocks, QUERY_THREADS, 0, st>>>(a);
  } else if (a.k <= 32) {
    apply_carveout<32>(k_query_packet<M, D, 32>);
    k_query_packet<M, D, 32><<<blocks, QUERY_THREADS, 0, st>>>(a);
  } else {
    constexpr size_t smem = sizeof(PacketSmem<64>);
    KD_TRY_CUDA(cudaFuncSetAttribute(k_query_packet_dyn<M, D, 64>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                     static_cast<int>(smem)));
    k_query_packet_dyn<M, D, 64><<<blocks, QUERY_THREADS, smem, st>>>(a);
  }
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
  return metric != M_LP && !use_eps && k >= 1 && k <= 64 && n_points < 0xffffffffull &&
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

#ifdef KD_WORK_COUNTS
// The packet traversal's work counters (kd_query_packet.cuh), added up since
// the last reset: out[0 .. n) (n <= 16); reset != 0 zeroes them afterwards.
extern "C" int kd_work_counts(unsigned long long* out, int n, int reset) {
  if (n < 0 || n > 16) return 1;
  unsigned long long h[16] = {};
  if (cudaDeviceSynchronize() != cudaSuccess || cudaMemcpyFromSymbol(h, kd::g_work, sizeof(h)) != cudaSuccess)
    return 2;
  for (int i = 0; i < n; ++i) out[i] = h[i];
  if (reset) {
    const unsigned long long z[16] = {};
    if (cudaMemcpyToSymbol(kd::g_work, z, sizeof(z)) != cudaSuccess) return 2;
  }
  return 0;
}
#endif
