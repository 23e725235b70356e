// GPU FP64 brute force over a block of rows: a subsample oracle at sizes
// where the CPU brute force cannot run.
//
// Reference counterpart: dumbBrute (src/kernel.cu:1243-1261), one thread per
// point against all points with the FP64 distance check.  Here one thread
// owns a query row i of [row0, row1) and counts the j != i with
// s(i, j) <= fl(eps*eps), s the reference predicate (src/utils.cu:296-309:
// sequential sum over the dimensions, subtraction, product and sum each
// rounded in FP64).  The candidate rows stream through shared memory in
// tiles that every thread of the block reads by broadcast.  The loop stops
// a pair as soon as the partial sum exceeds eps^2: adding non-negative
// rounded terms never decreases it, so the decision is unchanged.
#include "internal.cuh"

namespace mistic {
namespace {

constexpr int BR_THREADS = 256;

template <class T>
__global__ void __launch_bounds__(BR_THREADS) k_brute_rows(const T* __restrict__ X, uint64_t n, uint32_t d,
                                                           double eps2, uint64_t row0, uint64_t row1, uint32_t tile,
                                                           uint32_t* __restrict__ counts) {
  extern __shared__ double br_tile[];  // tile x d candidate rows, widened to FP64
  const uint64_t i = row0 + (uint64_t)blockIdx.x * BR_THREADS + threadIdx.x;
  const bool active = i < row1;
  const T* xi = X + (active ? i : row0) * d;
  uint32_t cnt = 0;
  for (uint64_t c0 = 0; c0 < n; c0 += tile) {
    const uint32_t m = (uint32_t)(n - c0 < (uint64_t)tile ? n - c0 : (uint64_t)tile);
    __syncthreads();
    for (uint32_t t = threadIdx.x; t < m * d; t += BR_THREADS) br_tile[t] = (double)X[c0 * d + t];
    __syncthreads();
    if (!active) continue;
    for (uint32_t j = 0; j < m; ++j) {
      if (c0 + j == i) continue;
      const double* xj = br_tile + (size_t)j * d;
      double s = 0.0;
      uint32_t t = 0;
      for (; t < d; ++t) {
        const double df = __dsub_rn((double)xi[t], xj[t]);
        s = __dadd_rn(s, __dmul_rn(df, df));
        if (s > eps2) break;
      }
      cnt += t == d ? 1u : 0u;
    }
  }
  if (active) counts[i - row0] = cnt;
}

}  // namespace

void bruteforce_rows(mistic_handle_s* h, const void* x, mistic_dtype dt, uint64_t n, uint32_t d, double eps2,
                     uint64_t row0, uint64_t row1, uint32_t* counts) {
  if (row1 <= row0) return;
  const uint32_t tile = (uint32_t)std::max<uint64_t>(1, std::min<uint64_t>(256, (32 * 1024) / (8ull * d)));
  const size_t smem = (size_t)tile * d * sizeof(double);
  const unsigned grid = (unsigned)((row1 - row0 + BR_THREADS - 1) / BR_THREADS);
  if (dt == MISTIC_F64) {
    k_brute_rows<double><<<grid, BR_THREADS, smem, h->stream>>>((const double*)x, n, d, eps2, row0, row1, tile,
                                                                 counts);
  } else {
    k_brute_rows<float><<<grid, BR_THREADS, smem, h->stream>>>((const float*)x, n, d, eps2, row0, row1, tile,
                                                                counts);
  }
  launched(h, "brute_rows");
}

}  // namespace mistic
