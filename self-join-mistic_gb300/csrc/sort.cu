// Device exclusive scan and LSD radix sort of 64-bit bin keys.
//
// The reference sorts with thrust (host `thrust::omp` sorts of bin numbers in
// src/nodes.cu:372,505 and device `sort_by_key` of result pairs in
// src/launcher.cu:3468,3488).  Here the bin keys of all n points are sorted
// once on the device: 8-bit digits, one histogram pass and one stable scatter
// pass per digit, only over the bits the packed key actually uses.
//
// Scatter ranking: each warp owns a contiguous run of 512 elements and ranks
// them 32 at a time with __match_any_sync, keeping per-warp digit counters in
// shared memory; a per-digit prefix over the 8 warps then gives every
// element its position inside the tile, and the digit-major scan of the
// per-tile histograms gives the tile's global base.  Element order within a
// digit is preserved (stable), which LSD sorting requires.
#include "internal.cuh"

namespace mistic {

// ------------------------------------------------------------------ scan

constexpr int SCAN_THREADS = 256;
constexpr int SCAN_ITEMS = 8;
constexpr int SCAN_TILE = SCAN_THREADS * SCAN_ITEMS;

template <class T>
__device__ __forceinline__ T warp_inclusive_scan(T x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    T y = __shfl_up_sync(FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Block-wide exclusive scan of one value per thread; `total` (optional)
// receives the block sum.  `ws` is 32 elements of shared scratch.
template <class T>
__device__ T block_exclusive_scan(T v, T* total, T* ws) {
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5, nw = blockDim.x >> 5;
  T x = warp_inclusive_scan(v);
  if (lane == 31) ws[w] = x;
  __syncthreads();
  if (w == 0) {
    T s = lane < nw ? ws[lane] : T(0);
    s = warp_inclusive_scan(s);
    if (lane < nw) ws[lane] = s;
  }
  __syncthreads();
  T prefix = w ? ws[w - 1] : T(0);
  if (total) *total = ws[nw - 1];
  __syncthreads();
  return prefix + x - v;
}

template <class T>
__global__ void k_scan_reduce(const T* __restrict__ in, size_t n, T* __restrict__ partial) {
  __shared__ T ws[32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  T s = 0;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    size_t idx = base + i;
    if (idx < n) s += in[idx];
  }
  T tot;
  block_exclusive_scan(s, &tot, ws);
  if (threadIdx.x == 0) partial[blockIdx.x] = tot;
}

template <class T>
__global__ void k_scan_partials(T* partial, size_t nb, T* total_out) {
  __shared__ T ws[32];
  T carry = 0;
  for (size_t c = 0; c < nb; c += blockDim.x) {
    size_t i = c + threadIdx.x;
    T v = i < nb ? partial[i] : T(0);
    T tot;
    T ex = block_exclusive_scan(v, &tot, ws);
    if (i < nb) partial[i] = carry + ex;
    carry += tot;
  }
  if (threadIdx.x == 0 && total_out) *total_out = carry;
}

template <class T>
__global__ void k_scan_down(const T* in, T* out, size_t n, const T* __restrict__ partial) {
  __shared__ T tile[SCAN_TILE];
  __shared__ T ws[32];
  const size_t base = (size_t)blockIdx.x * SCAN_TILE;
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    size_t idx = base + i;
    tile[i] = idx < n ? in[idx] : T(0);
  }
  __syncthreads();
  T loc[SCAN_ITEMS];
  T s = 0;
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    loc[j] = tile[threadIdx.x * SCAN_ITEMS + j];
    s += loc[j];
  }
  T run = block_exclusive_scan(s, (T*)nullptr, ws) + partial[blockIdx.x];
#pragma unroll
  for (int j = 0; j < SCAN_ITEMS; ++j) {
    tile[threadIdx.x * SCAN_ITEMS + j] = run;
    run += loc[j];
  }
  __syncthreads();
  for (int i = threadIdx.x; i < SCAN_TILE; i += SCAN_THREADS) {
    size_t idx = base + i;
    if (idx < n) out[idx] = tile[i];
  }
}

size_t scan_partials_count(size_t n) { return (n + SCAN_TILE - 1) / SCAN_TILE; }

template <class T>
void exclusive_scan(mistic_handle_s* h, const T* in, T* out, size_t n, T* total_dev) {
  if (n == 0) {
    if (total_dev) MCK(cudaMemsetAsync(total_dev, 0, sizeof(T), h->stream));
    return;
  }
  const size_t nb = scan_partials_count(n);
  T* partial = (T*)h->arena.get(sizeof(T) == 8 ? "scan_partial64" : "scan_partial32",
                                (nb + 1) * sizeof(T));
  k_scan_reduce<T><<<(unsigned)nb, SCAN_THREADS, 0, h->stream>>>(in, n, partial);
  launched(h, "scan_reduce");
  k_scan_partials<T><<<1, 1024, 0, h->stream>>>(partial, nb, total_dev);
  launched(h, "scan_partials");
  k_scan_down<T><<<(unsigned)nb, SCAN_THREADS, 0, h->stream>>>(in, out, n, partial);
  launched(h, "scan_down");
}

template void exclusive_scan<uint32_t>(mistic_handle_s*, const uint32_t*, uint32_t*, size_t, uint32_t*);
template void exclusive_scan<unsigned long long>(mistic_handle_s*, const unsigned long long*,
                                                 unsigned long long*, size_t, unsigned long long*);

// ------------------------------------------------------------------ radix sort

constexpr int RS_THREADS = 256;
constexpr int RS_WARPS = RS_THREADS / 32;
constexpr int RS_ROUNDS = 16;                        // 32-element rounds per warp
constexpr int RS_TILE = RS_THREADS * RS_ROUNDS;      // 4096 elements per block
constexpr int RS_BINS = 256;

__global__ void k_rs_hist(const uint64_t* __restrict__ keys, size_t n, int shift,
                          uint32_t* __restrict__ hist, uint32_t tiles) {
  __shared__ uint32_t cnt[RS_BINS];
  cnt[threadIdx.x] = 0;
  __syncthreads();
  const size_t base = (size_t)blockIdx.x * RS_TILE;
  for (int i = threadIdx.x; i < RS_TILE; i += RS_THREADS) {
    size_t idx = base + i;
    if (idx < n) atomicAdd(&cnt[(keys[idx] >> shift) & 0xff], 1u);
  }
  __syncthreads();
  hist[(size_t)threadIdx.x * tiles + blockIdx.x] = cnt[threadIdx.x];
}

template <bool HAS_VALS, bool IOTA>
__global__ void __launch_bounds__(RS_THREADS)
k_rs_scatter(const uint64_t* __restrict__ kin, const uint32_t* __restrict__ vin,
             uint64_t* __restrict__ kout, uint32_t* __restrict__ vout, size_t n,
             int shift, const uint32_t* __restrict__ offs, uint32_t tiles) {
  __shared__ uint32_t wcnt[RS_WARPS][RS_BINS];
  for (int i = threadIdx.x; i < RS_WARPS * RS_BINS; i += RS_THREADS) (&wcnt[0][0])[i] = 0;
  __syncthreads();
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const unsigned lt_mask = (1u << lane) - 1u;
  const size_t base = (size_t)blockIdx.x * RS_TILE + (size_t)w * (RS_ROUNDS * 32);
  uint64_t key[RS_ROUNDS];
  uint32_t val[RS_ROUNDS];
  uint32_t rank[RS_ROUNDS];
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const size_t idx = base + r * 32 + lane;
    const bool valid = idx < n;
    key[r] = valid ? kin[idx] : 0ull;
    if (HAS_VALS) val[r] = valid ? (IOTA ? (uint32_t)idx : vin[idx]) : 0u;
    // out-of-range lanes get a private sentinel digit so they match nobody
    const uint32_t dg = valid ? (uint32_t)((key[r] >> shift) & 0xff) : (RS_BINS + lane);
    const unsigned peers = __match_any_sync(FULL_MASK, dg);
    const uint32_t before = valid ? wcnt[w][dg] : 0u;
    __syncwarp();
    const uint32_t lt = __popc(peers & lt_mask);
    if (valid && lt == 0) wcnt[w][dg] = before + __popc(peers);
    __syncwarp();
    rank[r] = before + lt;
  }
  __syncthreads();
  {
    // exclusive prefix across warps, one digit per thread
    const int dgt = threadIdx.x;
    uint32_t run = 0;
#pragma unroll
    for (int ww = 0; ww < RS_WARPS; ++ww) {
      uint32_t c = wcnt[ww][dgt];
      wcnt[ww][dgt] = run;
      run += c;
    }
  }
  __syncthreads();
#pragma unroll
  for (int r = 0; r < RS_ROUNDS; ++r) {
    const size_t idx = base + r * 32 + lane;
    if (idx < n) {
      const uint32_t dg = (uint32_t)((key[r] >> shift) & 0xff);
      const size_t pos = (size_t)offs[(size_t)dg * tiles + blockIdx.x] + wcnt[w][dg] + rank[r];
      kout[pos] = key[r];
      if (HAS_VALS) vout[pos] = val[r];
    }
  }
}

int radix_sort_u64(mistic_handle_s* h, uint64_t* keys[2], uint32_t* vals[2], bool has_vals,
                   bool iota_vals, size_t n, int bits) {
  if (n <= 1 || bits <= 0) {
    if (n == 1 && has_vals && iota_vals) MCK(cudaMemsetAsync(vals[0], 0, sizeof(uint32_t), h->stream));
    return 0;
  }
  if (n > 0xffffffffull) throw Error(MISTIC_ERR_TOO_LARGE, "radix sort supports < 2^32 elements");
  const uint32_t tiles = (uint32_t)((n + RS_TILE - 1) / RS_TILE);
  uint32_t* hist = (uint32_t*)h->arena.get("rs_hist", (size_t)RS_BINS * tiles * sizeof(uint32_t));
  int cur = 0;
  bool first = true;
  for (int shift = 0; shift < bits; shift += 8) {
    k_rs_hist<<<tiles, RS_THREADS, 0, h->stream>>>(keys[cur], n, shift, hist, tiles);
    launched(h, "rs_hist");
    exclusive_scan<uint32_t>(h, hist, hist, (size_t)RS_BINS * tiles, nullptr);
    if (!has_vals) {
      k_rs_scatter<false, false><<<tiles, RS_THREADS, 0, h->stream>>>(
          keys[cur], nullptr, keys[cur ^ 1], nullptr, n, shift, hist, tiles);
    } else if (first && iota_vals) {
      k_rs_scatter<true, true><<<tiles, RS_THREADS, 0, h->stream>>>(
          keys[cur], nullptr, keys[cur ^ 1], vals[cur ^ 1], n, shift, hist, tiles);
    } else {
      k_rs_scatter<true, false><<<tiles, RS_THREADS, 0, h->stream>>>(
          keys[cur], vals[cur], keys[cur ^ 1], vals[cur ^ 1], n, shift, hist, tiles);
    }
    launched(h, "rs_scatter");
    cur ^= 1;
    first = false;
  }
  return cur;
}

}  // namespace mistic
