// Reference-point bin index and neighbour-bin enumeration on the device.
//
// Reference counterparts (bwd29/self-join-MiSTIC):
//  - binningKernel, src/kernel.cu:880-909: per point, floor(||x - r|| / ε)
//    for each reference point in FP64.  Here the same FP64 distances are
//    taken to k reference points and quantised with a width slightly above ε
//    so the triangle-inequality argument survives rounding (see k_pack_keys).
//  - the host-built node net, src/nodes.cu:5-356, whose neighbour relation is
//    "bins differ by at most one on every layer" (src/nodes.cu:416-435,
//    719-747).  Here the bin keys are packed into one 64-bit key, radix
//    sorted, and non-empty bins become contiguous runs of the sorted order.
//  - the 3^k neighbour search over sorted bin keys, generateRanges /
//    binarySearch in src/tree.cu:596-759,886-996 (device form
//    GPUBinarySearch, src/kernel.cu:164-224).  Here one thread per non-empty
//    bin walks the ±1 neighbourhood depth-first, narrowing a sorted range one
//    key field at a time (the top fields through a direct-address prefix
//    table), so empty prefixes are pruned early; only neighbours of index >=
//    the home bin are emitted (each unordered bin pair once).
#include <math.h>

#include "internal.cuh"

namespace mistic {

template <class T>
__device__ __forceinline__ double ld(const T* p, size_t i) {
  return (double)p[i];
}

// ------------------------------------------------------------ column stats
// Per-column min, max and sum over all rows plus a finiteness flag.  Each
// block writes its partials; a second kernel folds them in a fixed order so
// the result (and therefore the reference points) is deterministic.

constexpr int CS_ROWS = 8;

template <class T>
__global__ void k_colstats(const T* __restrict__ x, size_t n, uint32_t d, double* __restrict__ part,
                           unsigned* __restrict__ nonfinite) {
  // part layout: [blockIdx.y][3][d] : min, max, sum for the block's rows of column tile blockIdx.x
  __shared__ double smin[CS_ROWS][32], smax[CS_ROWS][32], ssum[CS_ROWS][32];
  const uint32_t col = blockIdx.x * 32 + threadIdx.x;
  double mn = INFINITY, mx = -INFINITY, sm = 0.0;
  bool bad = false;
  if (col < d) {
    for (size_t r = (size_t)blockIdx.y * CS_ROWS + threadIdx.y; r < n; r += (size_t)gridDim.y * CS_ROWS) {
      double v = ld(x, r * d + col);
      if (!isfinite(v)) bad = true;
      mn = fmin(mn, v);
      mx = fmax(mx, v);
      sm += v;
    }
  }
  if (bad) atomicOr(nonfinite, 1u);
  smin[threadIdx.y][threadIdx.x] = mn;
  smax[threadIdx.y][threadIdx.x] = mx;
  ssum[threadIdx.y][threadIdx.x] = sm;
  __syncthreads();
  if (threadIdx.y == 0 && col < d) {
    for (int r = 1; r < CS_ROWS; ++r) {
      mn = fmin(mn, smin[r][threadIdx.x]);
      mx = fmax(mx, smax[r][threadIdx.x]);
      sm += ssum[r][threadIdx.x];
    }
    double* p = part + (size_t)blockIdx.y * 3 * d;
    p[col] = mn;
    p[d + col] = mx;
    p[2 * d + col] = sm;
  }
}

__global__ void k_colstats_final(const double* __restrict__ part, uint32_t nparts, uint32_t d,
                                 size_t n, double* __restrict__ out /* mean, min, max */) {
  const uint32_t col = blockIdx.x * blockDim.x + threadIdx.x;
  if (col >= d) return;
  double mn = INFINITY, mx = -INFINITY, sm = 0.0;
  for (uint32_t b = 0; b < nparts; ++b) {
    const double* p = part + (size_t)b * 3 * d;
    mn = fmin(mn, p[col]);
    mx = fmax(mx, p[d + col]);
    sm += p[2 * d + col];
  }
  out[col] = n ? sm / (double)n : 0.0;
  out[d + col] = mn;
  out[2 * d + col] = mx;
}

// ------------------------------------------------------------ sample covariance
template <class T>
__global__ void k_gather_sample(const T* __restrict__ x, size_t n, uint32_t d, uint32_t S,
                                double* __restrict__ s) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)S * d) return;
  const size_t row = i / d, col = i % d;
  const size_t src = (size_t)((row * (unsigned long long)n) / S);
  s[i] = ld(x, src * d + col);
}

// Sample covariance about the full-data mean mu: each block accumulates a
// 16 x 16 tile of (a, b) over one chunk of sample rows (staged in shared
// memory); a second kernel adds the chunk partials in a fixed order, so the
// result - and the reference points derived from it - is deterministic.
constexpr int COV_T = 16;
constexpr int COV_CHUNK = 128;

__global__ void k_sample_cov_part(const double* __restrict__ s, uint32_t S, uint32_t d, const double* __restrict__ mu,
                                  double* __restrict__ part /* [chunks][d][d] */) {
  __shared__ double sa[COV_CHUNK][COV_T + 1], sb[COV_CHUNK][COV_T + 1];
  const uint32_t a0 = blockIdx.y * COV_T, b0 = blockIdx.x * COV_T, r0 = blockIdx.z * COV_CHUNK;
  const int tx = threadIdx.x, ty = threadIdx.y, t = ty * COV_T + tx;
  for (int i = t; i < COV_CHUNK * COV_T; i += COV_T * COV_T) {
    const int rr = i / COV_T, cc = i % COV_T;
    const uint32_t row = r0 + rr;
    double va = 0.0, vb = 0.0;
    if (row < S && a0 + cc < d) va = s[(size_t)row * d + a0 + cc] - mu[a0 + cc];
    if (row < S && b0 + cc < d) vb = s[(size_t)row * d + b0 + cc] - mu[b0 + cc];
    sa[rr][cc] = va;
    sb[rr][cc] = vb;
  }
  __syncthreads();
  double acc = 0.0;
  for (int rr = 0; rr < COV_CHUNK; ++rr) acc = fma(sa[rr][ty], sb[rr][tx], acc);
  const uint32_t a = a0 + ty, b = b0 + tx;
  if (a < d && b < d) part[((size_t)blockIdx.z * d + a) * d + b] = acc;
}

__global__ void k_sample_cov_final(const double* __restrict__ part, uint32_t chunks, uint32_t d, uint32_t S,
                                   double* __restrict__ cov) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= (size_t)d * d) return;
  double acc = 0.0;
  for (uint32_t c = 0; c < chunks; ++c) acc += part[(size_t)c * d * d + i];
  cov[i] = acc / S;
}

// ------------------------------------------------------------ reference-point distances
// D[i][j] = FP64 ||x_i - r_j|| (sequential sum, then sqrt), with per-block
// min/max partials per reference point.
constexpr int RPD_THREADS = 256;
constexpr uint32_t RPD_DMAX = 48;  // rows staged in shared memory up to this d

template <class T>
__global__ void __launch_bounds__(RPD_THREADS)
k_rp_dist(const T* __restrict__ x, size_t n, uint32_t d, const double* __restrict__ rps, int k,
          double* __restrict__ D, double* __restrict__ part /* [block][2][k] */) {
  // dynamic shared memory: k x d reference points, then a tile of rows
  // (RPD_THREADS rows of up to RPD_DMAX coordinates) copied with coalesced loads
  extern __shared__ double srp[];
  double* tile = srp + (size_t)k * d;
  for (uint32_t i = threadIdx.x; i < (uint32_t)k * d; i += blockDim.x) srp[i] = rps[i];
  __shared__ double smn[MAX_K][RPD_THREADS / 32], smx[MAX_K][RPD_THREADS / 32];
  const size_t row0 = (size_t)blockIdx.x * blockDim.x;
  const uint32_t rows = (uint32_t)min((size_t)blockDim.x, n > row0 ? n - row0 : 0);
  const bool staged = d <= RPD_DMAX;
  if (staged) {
    const size_t base = row0 * d;
    for (uint32_t i = threadIdx.x; i < rows * d; i += blockDim.x) tile[i] = (double)x[base + i];
  }
  __syncthreads();
  const size_t i = row0 + threadIdx.x;
  const bool valid = i < n;
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  for (int j = 0; j < k; ++j) {
    double dist = 0.0;
    if (valid) {
      double s = 0.0;
      const double* r = srp + (size_t)j * d;
      for (uint32_t t = 0; t < d; ++t) {
        const double xv = staged ? tile[(size_t)threadIdx.x * d + t] : (double)x[i * d + t];
        const double df = xv - r[t];
        s = fma(df, df, s);
      }
      dist = sqrt(s);
      D[i * k + j] = dist;
    }
    double mn = valid ? dist : INFINITY, mx = valid ? dist : -INFINITY;
#pragma unroll
    for (int o = 16; o; o >>= 1) {
      mn = fmin(mn, __shfl_xor_sync(FULL_MASK, mn, o));
      mx = fmax(mx, __shfl_xor_sync(FULL_MASK, mx, o));
    }
    if (lane == 0) {
      smn[j][w] = mn;
      smx[j][w] = mx;
    }
  }
  __syncthreads();
  if (threadIdx.x < (unsigned)k) {
    const int j = threadIdx.x;
    double mn = INFINITY, mx = -INFINITY;
    for (int ww = 0; ww < RPD_THREADS / 32; ++ww) {
      mn = fmin(mn, smn[j][ww]);
      mx = fmax(mx, smx[j][ww]);
    }
    part[(size_t)blockIdx.x * 2 * k + j] = mn;
    part[(size_t)blockIdx.x * 2 * k + k + j] = mx;
  }
}

__global__ void k_minmax_final(const double* __restrict__ part, uint32_t nparts, int k,
                               double* __restrict__ out /* min[k], max[k] */) {
  // one block per reference point; fixed reduction order (deterministic)
  const int j = blockIdx.x;
  double mn = INFINITY, mx = -INFINITY;
  for (uint32_t b = threadIdx.x; b < nparts; b += blockDim.x) {
    mn = fmin(mn, part[(size_t)b * 2 * k + j]);
    mx = fmax(mx, part[(size_t)b * 2 * k + k + j]);
  }
  __shared__ double smn[32], smx[32];
#pragma unroll
  for (int o = 16; o; o >>= 1) {
    mn = fmin(mn, __shfl_xor_sync(FULL_MASK, mn, o));
    mx = fmax(mx, __shfl_xor_sync(FULL_MASK, mx, o));
  }
  if ((threadIdx.x & 31) == 0) {
    smn[threadIdx.x >> 5] = mn;
    smx[threadIdx.x >> 5] = mx;
  }
  __syncthreads();
  if (threadIdx.x == 0) {
    for (int w = 1; w < (int)(blockDim.x >> 5); ++w) {
      mn = fmin(mn, smn[w]);
      mx = fmax(mx, smx[w]);
    }
    out[j] = mn;
    out[k + j] = mx;
  }
}

// ------------------------------------------------------------ key packing
// field_j = floor((D_ij - Dmin_j) / w_j), clamped to [0, maxkey_j].
// Completeness: for any pair in the result, |D_xj - D_yj| (computed) is
// below w_j, so the two fields differ by at most one; w_j = ε(1+δ) with δ
// covering the FP64 rounding of the distances and of the quotient (chosen
// on the host).  Clamping only shrinks differences.
__global__ void k_pack_keys(const double* __restrict__ D, size_t n, PackParams P,
                            uint64_t* __restrict__ keys) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  uint64_t key = 0;
  for (int j = 0; j < P.k; ++j) {
    double v = floor((D[i * P.kstride + P.col[j]] - P.dmin[j]) / P.w[j]);
    v = fmin(fmax(v, 0.0), (double)P.maxkey[j]);
    key |= (uint64_t)v << P.shift[j];
  }
  keys[i] = key;
}

__global__ void k_iota(uint32_t* v, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = (uint32_t)i;
}

// ------------------------------------------------------------ bins
__global__ void k_bin_flags(const uint64_t* __restrict__ keys, size_t n, uint32_t* __restrict__ flags) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  flags[i] = (i == 0 || keys[i] != keys[i - 1]) ? 1u : 0u;
}

__global__ void k_bin_starts(const uint64_t* __restrict__ keys, size_t n,
                             const uint32_t* __restrict__ binid /* exclusive scan of flags */,
                             uint32_t* __restrict__ bstart, uint64_t* __restrict__ bkey) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const bool head = (i == 0 || keys[i] != keys[i - 1]);
  if (head) {
    bstart[binid[i]] = (uint32_t)i;
    bkey[binid[i]] = keys[i];
  }
  if (i == n - 1) bstart[binid[i] + (head ? 1 : 0)] = (uint32_t)n;
}

// ------------------------------------------------------------ point gather
// Sorted-order copies for the join: FP32 centred coordinates (row stride
// dpad, zero padded), the original row ids, and optionally FP64 rows for the
// plain FP64 join.  Also the largest FP32 row norm (for the filter's error
// bound), reduced per block.
template <class T>
__global__ void k_gather_points(const T* __restrict__ x, size_t n, uint32_t d,
                                const uint32_t* __restrict__ perm, const double* __restrict__ center,
                                uint32_t dpad32, float* __restrict__ xf, uint32_t dpad64,
                                double* __restrict__ xd, uint32_t* __restrict__ ids,
                                double* __restrict__ norm_part) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  double nrm2 = 0.0;
  if (p < n) {
    const uint32_t src = perm[p];
    ids[p] = src;
    for (uint32_t t = 0; t < dpad32; ++t) {
      float v = 0.f;
      if (t < d) v = (float)(ld(x, (size_t)src * d + t) - center[t]);
      if (xf) xf[p * dpad32 + t] = v;
      nrm2 = fma((double)v, (double)v, nrm2);
    }
    if (xd) {
      for (uint32_t t = 0; t < dpad64; ++t) xd[p * dpad64 + t] = t < d ? ld(x, (size_t)src * d + t) : 0.0;
    }
  }
  // block max of nrm2
#pragma unroll
  for (int o = 16; o; o >>= 1) nrm2 = fmax(nrm2, __shfl_xor_sync(FULL_MASK, nrm2, o));
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = nrm2;
  __syncthreads();
  if (threadIdx.x == 0) {
    double m = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) m = fmax(m, sm[w]);
    norm_part[blockIdx.x] = m;
  }
}

__global__ void k_max_final(const double* __restrict__ part, uint32_t nparts, double* out) {
  double m = 0;
  for (uint32_t i = threadIdx.x; i < nparts; i += blockDim.x) m = fmax(m, part[i]);
#pragma unroll
  for (int o = 16; o; o >>= 1) m = fmax(m, __shfl_xor_sync(FULL_MASK, m, o));
  __shared__ double sm[32];
  if ((threadIdx.x & 31) == 0) sm[threadIdx.x >> 5] = m;
  __syncthreads();
  if (threadIdx.x == 0) {
    double r = 0;
    for (int w = 0; w < (int)(blockDim.x >> 5); ++w) r = fmax(r, sm[w]);
    *out = r;
  }
}

// ------------------------------------------------------------ neighbour enumeration
// One thread per non-empty bin h.  Depth-first over the key fields: at
// level j the candidate field value is K_j - 1, K_j, K_j + 1; the bins whose
// key starts with the chosen prefix form a contiguous sorted range, found by
// two lower-bound searches inside the parent range.  The first p fields
// skip the searches: a direct-address table (ptab[v] = first bin whose
// p-field prefix, read as a mixed-radix number, is >= v) gives the range of
// each of the 3^p prefixes with two loads, and the walk starts at level p
// inside it.  A range lying wholly below h is skipped (home <= neighbour).
// Leaves come out in ascending bin order, starting with h itself.
//
// Pass 1 (fill == false) counts neighbours, join work units and candidate
// pairs per home bin; pass 2 writes the neighbour list and the units.  The
// neighbour list of h is cut into segments of about `seg_cap` candidate
// points, and the home bin into chunks of `chunk` points; one unit is one
// (chunk, segment) combination.
__device__ __forceinline__ uint32_t lower_bound_u64(const uint64_t* __restrict__ a, uint32_t lo,
                                                    uint32_t hi, uint64_t v) {
  while (lo < hi) {
    uint32_t mid = lo + ((hi - lo) >> 1);
    if (a[mid] < v)
      lo = mid + 1;
    else
      hi = mid;
  }
  return lo;
}

// Home-point sample (mistic_opts.home_sample): group g (points
// [512 g, 512 g + 512) of bin h's sorted order) takes part iff a hash of
// (h, g) is 0 mod S.  Every unit chunk size (4 .. 512 points) divides 512,
// so a unit is either wholly in the sample or wholly out of it, in every mode.
constexpr uint32_t SAMPLE_GROUP = 512;
__device__ __forceinline__ bool group_sampled(uint32_t h, uint32_t g, uint32_t S) {
  if (S <= 1) return true;
  uint32_t x = h * 0x9E3779B1u ^ (g + 0x7F4A7C15u) * 0x85EBCA77u;
  x ^= x >> 15;
  x *= 0x2C1B3C6Du;
  x ^= x >> 12;
  return x % S == 0;
}

// Field j of key K: bits [shift[j], shift[j-1]) (shift[-1] = 64).
__device__ __forceinline__ int key_field(uint64_t K, const EnumParams& P, int j) {
  const int hi_bit = j == 0 ? 64 : P.shift[j - 1];
  const int width = hi_bit - P.shift[j];
  const uint64_t mask = width >= 64 ? ~0ull : ((1ull << width) - 1ull);
  return (int)((K >> P.shift[j]) & mask);
}

// The same walk for any depth, with its per-level state in arrays (local
// memory): used below the levels walk_levels keeps in registers.
template <class Leaf>
__device__ __noinline__ void walk_deep(const uint64_t* __restrict__ bkey, uint64_t K, uint32_t hb,
                                       const EnumParams& P, int j0, uint32_t lo0, uint32_t hi0, uint64_t base0,
                                       Leaf& leaf) {
  uint32_t lo[MAX_K + 1], hi[MAX_K + 1];
  uint64_t base[MAX_K + 1];
  int di[MAX_K + 1];
  lo[j0] = lo0;
  hi[j0] = hi0;
  base[j0] = base0;
  di[j0] = 0;
  int j = j0;
  while (j >= j0) {
    if (di[j] == 3) {
      --j;
      if (j >= j0) ++di[j];
      continue;
    }
    const int cv = key_field(K, P, j) + di[j] - 1;
    if (cv < 0 || (long long)cv > (long long)P.maxkey[j]) {
      ++di[j];
      continue;
    }
    const uint64_t lower = base[j] | ((uint64_t)cv << P.shift[j]);
    const uint64_t upper = lower + (1ull << P.shift[j]);
    const uint32_t a = lower_bound_u64(bkey, lo[j], hi[j], lower);
    const uint32_t b = lower_bound_u64(bkey, a, hi[j], upper);
    if (a == b || b <= hb) {
      ++di[j];
      continue;
    }
    if (j == P.k - 1) {
      leaf(a);
      ++di[j];
      continue;
    }
    base[j + 1] = lower;
    lo[j + 1] = a;
    hi[j + 1] = b;
    di[j + 1] = 0;
    ++j;
  }
}

// Depth-first walk of key fields j .. k-1 of home key K inside the sorted bin
// range [lo, hi) whose keys share the prefix bits `base`: field values
// K_j - 1, K_j, K_j + 1 in order, each narrowed by two lower-bound searches;
// leaf(a) for every bin a >= hb, in ascending order.  The first R levels
// keep their range and loop state in registers; deeper ones go to walk_deep.
template <int R, class Leaf>
__device__ __forceinline__ void walk_levels(const uint64_t* __restrict__ bkey, uint64_t K, uint32_t hb,
                                            const EnumParams& P, int j, uint32_t lo, uint32_t hi, uint64_t base,
                                            Leaf& leaf) {
  const int sh = P.shift[j];
  const int kfj = key_field(K, P, j);
#pragma unroll 1
  for (int di = 0; di < 3; ++di) {
    const int cv = kfj + di - 1;
    if (cv < 0 || (long long)cv > (long long)P.maxkey[j]) continue;
    const uint64_t lower = base | ((uint64_t)cv << sh);
    const uint64_t upper = lower + (1ull << sh);
    const uint32_t a = lower_bound_u64(bkey, lo, hi, lower);
    const uint32_t b = lower_bound_u64(bkey, a, hi, upper);
    if (a == b || b <= hb) continue;
    if (j == P.k - 1) {
      leaf(a);  // b == a + 1 and a >= hb
      continue;
    }
    if constexpr (R > 1)
      walk_levels<R - 1>(bkey, K, hb, P, j + 1, a, b, lower, leaf);
    else
      walk_deep(bkey, K, hb, P, j + 1, a, b, lower, leaf);
  }
}

template <bool FILL>
__global__ void __launch_bounds__(128, 8) k_enum(const uint64_t* __restrict__ bkey, const uint32_t* __restrict__ bstart,
                       uint32_t m, EnumParams P, uint32_t* __restrict__ nbr_cnt,
                       uint32_t* __restrict__ unit_cnt, uint32_t* __restrict__ unit_cnt_tc,
                       unsigned long long* __restrict__ cand, const uint32_t* __restrict__ nbr_off,
                       const uint32_t* __restrict__ unit_off, const uint32_t* __restrict__ unit_off_tc,
                       uint32_t* __restrict__ nbr, Unit* __restrict__ units_simt, Unit* __restrict__ units_tc) {
  const uint32_t hb = blockIdx.x * blockDim.x + threadIdx.x;
  if (hb >= m) return;
  const uint64_t K = bkey[hb];
  const uint32_t asz = bstart[hb + 1] - bstart[hb];
  // large home bins go to the tensor-core join (128-row chunks), the rest to the CUDA-core join
  const bool tc = P.tc_min > 0 && asz >= P.tc_min;
  const uint32_t csz = tc ? P.tc_chunk : P.chunk;
  const uint32_t nchunks = (asz + csz - 1) / csz;
  Unit* __restrict__ units = tc ? units_tc : units_simt;
  // sampled home points: chunks taken, home points and their pairs inside the bin
  uint32_t nchunks_s = nchunks;
  unsigned long long rows_s = asz, self_s = (unsigned long long)asz * (asz - (asz > 0)) / 2;
  if (P.sample > 1) {
    nchunks_s = 0;
    for (uint32_t ch = 0; ch < nchunks; ++ch) nchunks_s += group_sampled(hb, ch * csz / SAMPLE_GROUP, P.sample);
    rows_s = 0;
    self_s = 0;
    for (uint32_t g0 = 0; g0 < asz; g0 += SAMPLE_GROUP) {
      if (!group_sampled(hb, g0 / SAMPLE_GROUP, P.sample)) continue;
      const unsigned long long g1 = min(asz, g0 + SAMPLE_GROUP), c = g1 - g0;
      rows_s += c;
      self_s += c * (asz - 1) - (g0 + g1 - 1) * c / 2;  // pairs (p, q) of the bin with p in the group, q > p
    }
  }


  uint32_t cnt = 0, nseg = 0, seg_fill = 0, seg_begin = 0;
  unsigned long long c = 0;
  uint32_t w_nbr = FILL ? nbr_off[hb] : 0;
  uint32_t w_unit = FILL ? (tc ? unit_off_tc[hb] : unit_off[hb]) : 0;

  // Visits neighbour bin `a` (ascending, a >= hb): candidate count, segment
  // split and, in pass 2, the neighbour list and the units.
  auto leaf = [&](uint32_t a) {
    const uint32_t bsz = bstart[a + 1] - bstart[a];
    c += (a == hb) ? self_s : rows_s * bsz;
    if (seg_fill > 0 && seg_fill + bsz > (tc ? P.seg_cap_tc : P.seg_cap)) {
      if (FILL) {
        for (uint32_t ch = 0; ch < nchunks; ++ch)
          if (group_sampled(hb, ch * csz / SAMPLE_GROUP, P.sample))
            units[w_unit++] = Unit{hb, ch, nbr_off[hb] + seg_begin, nbr_off[hb] + cnt};
      }
      ++nseg;
      seg_fill = 0;
      seg_begin = cnt;
    }
    seg_fill += bsz;
    if (FILL) nbr[w_nbr++] = a;
    ++cnt;
  };

  if (P.k == 0) {
    leaf(hb);  // no key fields: one bin holding every point
  } else if (P.p == 0) {
    walk_levels<3>(bkey, K, hb, P, 0, 0u, m, 0ull, leaf);
  } else {
    // prefixes in ascending order: field j offset by digit j of c in base 3
    // (field 0 most significant)
    uint32_t n3 = 1;
    for (int q = 0; q < P.p; ++q) n3 *= 3;
    for (uint32_t cb = 0; cb < n3; ++cb) {
      uint32_t rem = cb, pw = n3 / 3, idx = 0;
      uint64_t pre = 0;
      bool ok = true;
      for (int q = 0; q < P.p; ++q) {
        const uint32_t t = rem / pw;
        rem -= t * pw;
        pw /= 3;
        const int cv = key_field(K, P, q) + (int)t - 1;
        if (cv < 0 || (uint32_t)cv > P.maxkey[q]) {
          ok = false;
          break;
        }
        idx += (uint32_t)cv * P.stride[q];
        pre |= (uint64_t)cv << P.shift[q];
      }
      if (!ok) continue;
      const uint32_t r0 = P.ptab[idx], r1 = P.ptab[idx + 1];
      if (r0 == r1 || r1 <= hb) continue;
      if (P.p == P.k) {  // every field fixed: the single bin r0 (>= hb)
        leaf(r0);
        continue;
      }
      walk_levels<3>(bkey, K, hb, P, P.p, r0, r1, pre, leaf);
    }
  }
  if (cnt > 0) {
    if (FILL) {
      for (uint32_t ch = 0; ch < nchunks; ++ch)
        if (group_sampled(hb, ch * csz / SAMPLE_GROUP, P.sample))
          units[w_unit++] = Unit{hb, ch, nbr_off[hb] + seg_begin, nbr_off[hb] + cnt};
    }
    ++nseg;
  }
  if (!FILL) {
    // a bin's unit count saturates at 2^32 - 1; the 64-bit totals of the
    // three count arrays (k_count_totals) then exceed the 32-bit offsets the
    // work lists use, and the call fails with MISTIC_ERR_TOO_LARGE
    const unsigned long long nu = (unsigned long long)nseg * nchunks_s;
    const uint32_t nu32 = nu > 0xffffffffull ? 0xffffffffu : (uint32_t)nu;
    nbr_cnt[hb] = cnt;
    unit_cnt[hb] = tc ? 0u : nu32;
    unit_cnt_tc[hb] = tc ? nu32 : 0u;
    cand[hb] = c;
  }
}

// Bins per prefix of the enumeration table: cnt[v] += 1 for each bin whose
// first P.p key fields, as a mixed-radix number with strides P.stride, are v.
__global__ void k_prefix_count(const uint64_t* __restrict__ bkey, uint32_t m, EnumParams P,
                               uint32_t* __restrict__ cnt) {
  const uint32_t b = blockIdx.x * blockDim.x + threadIdx.x;
  if (b >= m) return;
  const uint64_t K = bkey[b];
  uint32_t v = 0;
  for (int j = 0; j < P.p; ++j) {
    const int w = min((j == 0 ? 64 : P.shift[j - 1]) - P.shift[j], 63);
    v += (uint32_t)((K >> P.shift[j]) & ((1ull << w) - 1ull)) * P.stride[j];
  }
  atomicAdd(&cnt[v], 1u);
}

// 64-bit sums of the three per-bin count arrays of the enumeration (the
// scans that turn them into offsets are 32-bit).
__global__ void k_count_totals(const uint32_t* __restrict__ a, const uint32_t* __restrict__ b,
                               const uint32_t* __restrict__ c, uint32_t m, unsigned long long* __restrict__ tot) {
  unsigned long long s[3] = {0, 0, 0};
  for (uint32_t i = blockIdx.x * blockDim.x + threadIdx.x; i < m; i += gridDim.x * blockDim.x) {
    s[0] += a[i];
    s[1] += b[i];
    s[2] += c[i];
  }
#pragma unroll
  for (int k = 0; k < 3; ++k) {
#pragma unroll
    for (int o = 16; o; o >>= 1) s[k] += __shfl_xor_sync(FULL_MASK, s[k], o);
  }
  if ((threadIdx.x & 31) == 0)
    for (int k = 0; k < 3; ++k)
      if (s[k]) atomicAdd(&tot[k], s[k]);
}

// ------------------------------------------------------------ host launchers
namespace idx {

void colstats(mistic_handle_s* h, const void* x, mistic_dtype dt, size_t n, uint32_t d,
              double* part, uint32_t nparts, double* out, unsigned* nonfinite) {
  dim3 blk(32, CS_ROWS), grd((d + 31) / 32, nparts);
  if (dt == MISTIC_F64)
    k_colstats<double><<<grd, blk, 0, h->stream>>>((const double*)x, n, d, part, nonfinite);
  else
    k_colstats<float><<<grd, blk, 0, h->stream>>>((const float*)x, n, d, part, nonfinite);
  launched(h, "colstats");
  k_colstats_final<<<(d + 127) / 128, 128, 0, h->stream>>>(part, nparts, d, n, out);
  launched(h, "colstats_final");
}

void sample_cov(mistic_handle_s* h, const void* x, mistic_dtype dt, size_t n, uint32_t d,
                uint32_t S, double* sbuf, const double* mu, double* part, double* cov) {
  const size_t tot = (size_t)S * d;
  const unsigned nb = (unsigned)((tot + 255) / 256);
  if (dt == MISTIC_F64)
    k_gather_sample<double><<<nb, 256, 0, h->stream>>>((const double*)x, n, d, S, sbuf);
  else
    k_gather_sample<float><<<nb, 256, 0, h->stream>>>((const float*)x, n, d, S, sbuf);
  launched(h, "gather_sample");
  const uint32_t chunks = (S + COV_CHUNK - 1) / COV_CHUNK;
  dim3 blk(COV_T, COV_T), grd((d + COV_T - 1) / COV_T, (d + COV_T - 1) / COV_T, chunks);
  k_sample_cov_part<<<grd, blk, 0, h->stream>>>(sbuf, S, d, mu, part);
  launched(h, "sample_cov_part");
  k_sample_cov_final<<<(unsigned)(((size_t)d * d + 255) / 256), 256, 0, h->stream>>>(part, chunks, d, S, cov);
  launched(h, "sample_cov_final");
}

void rp_dist(mistic_handle_s* h, const void* x, mistic_dtype dt, size_t n, uint32_t d,
             const double* rps, int k, double* D, double* part, uint32_t nparts, double* mm) {
  const size_t smem = (size_t)k * d * sizeof(double) + (d <= RPD_DMAX ? (size_t)RPD_THREADS * d * sizeof(double) : 0);
  if (dt == MISTIC_F64)  // the limit includes static shared memory: raise it whatever the size
    allow_max_dyn_smem(k_rp_dist<double>);
  else
    allow_max_dyn_smem(k_rp_dist<float>);
  if (dt == MISTIC_F64)
    k_rp_dist<double><<<nparts, RPD_THREADS, smem, h->stream>>>((const double*)x, n, d, rps, k, D, part);
  else
    k_rp_dist<float><<<nparts, RPD_THREADS, smem, h->stream>>>((const float*)x, n, d, rps, k, D, part);
  launched(h, "rp_dist");
  k_minmax_final<<<k, 256, 0, h->stream>>>(part, nparts, k, mm);
  launched(h, "minmax_final");
}

void pack_keys(mistic_handle_s* h, const double* D, size_t n, const PackParams& P, uint64_t* keys) {
  k_pack_keys<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(D, n, P, keys);
  launched(h, "pack_keys");
}

void iota(mistic_handle_s* h, uint32_t* v, size_t n) {
  k_iota<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(v, n);
  launched(h, "iota");
}

void bins(mistic_handle_s* h, const uint64_t* keys, size_t n, uint32_t* flags, uint32_t* nbins_dev,
          uint32_t* bstart, uint64_t* bkey) {
  const unsigned nb = (unsigned)((n + 255) / 256);
  k_bin_flags<<<nb, 256, 0, h->stream>>>(keys, n, flags);
  launched(h, "bin_flags");
  exclusive_scan<uint32_t>(h, flags, flags, n, nbins_dev);
  k_bin_starts<<<nb, 256, 0, h->stream>>>(keys, n, flags, bstart, bkey);
  launched(h, "bin_starts");
}

void gather(mistic_handle_s* h, const void* x, mistic_dtype dt, size_t n, uint32_t d,
            const uint32_t* perm, const double* center, uint32_t dpad32, float* xf, uint32_t dpad64,
            double* xd, uint32_t* ids, double* norm_part, double* rmax) {
  const unsigned nb = (unsigned)((n + 255) / 256);
  if (dt == MISTIC_F64)
    k_gather_points<double><<<nb, 256, 0, h->stream>>>((const double*)x, n, d, perm, center, dpad32, xf,
                                                      dpad64, xd, ids, norm_part);
  else
    k_gather_points<float><<<nb, 256, 0, h->stream>>>((const float*)x, n, d, perm, center, dpad32, xf,
                                                     dpad64, xd, ids, norm_part);
  launched(h, "gather_points");
  k_max_final<<<1, 1024, 0, h->stream>>>(norm_part, nb, rmax);
  launched(h, "max_final");
}

void prefix_table(mistic_handle_s* h, const uint64_t* bkey, uint32_t m, const EnumParams& P, uint32_t* ptab,
                  uint32_t entries) {
  MCK(cudaMemsetAsync(ptab, 0, ((size_t)entries + 1) * sizeof(uint32_t), h->stream));
  k_prefix_count<<<(m + 255) / 256, 256, 0, h->stream>>>(bkey, m, P, ptab);
  launched(h, "prefix_count");
  exclusive_scan<uint32_t>(h, ptab, ptab, (size_t)entries + 1, nullptr);
}

void enumerate(mistic_handle_s* h, const uint64_t* bkey, const uint32_t* bstart, uint32_t m,
               const EnumParams& P, uint32_t* nbr_cnt, uint32_t* unit_cnt, uint32_t* unit_cnt_tc,
               unsigned long long* cand, const uint32_t* nbr_off, const uint32_t* unit_off,
               const uint32_t* unit_off_tc, uint32_t* nbr, Unit* units, Unit* units_tc, bool fill) {
  const unsigned nb = (m + 127) / 128;
  if (!fill)
    k_enum<false><<<nb, 128, 0, h->stream>>>(bkey, bstart, m, P, nbr_cnt, unit_cnt, unit_cnt_tc, cand, nullptr,
                                             nullptr, nullptr, nullptr, nullptr, nullptr);
  else
    k_enum<true><<<nb, 128, 0, h->stream>>>(bkey, bstart, m, P, nullptr, nullptr, nullptr, nullptr, nbr_off,
                                            unit_off, unit_off_tc, nbr, units, units_tc);
  launched(h, fill ? "enum_fill" : "enum_count");
}

// Points per log2 bin-size class: hist[c] += size of every bin with
// floor(log2(size)) == c (c < 32).
__global__ void k_bin_hist(const uint32_t* __restrict__ bstart, uint32_t m, unsigned long long* __restrict__ hist) {
  __shared__ unsigned long long sh[32];
  if (threadIdx.x < 32) sh[threadIdx.x] = 0;
  __syncthreads();
  for (uint32_t b = blockIdx.x * blockDim.x + threadIdx.x; b < m; b += gridDim.x * blockDim.x) {
    const uint32_t sz = bstart[b + 1] - bstart[b];
    if (sz) atomicAdd(&sh[31 - __clz(sz)], (unsigned long long)sz);
  }
  __syncthreads();
  if (threadIdx.x < 32 && sh[threadIdx.x]) atomicAdd(&hist[threadIdx.x], sh[threadIdx.x]);
}

void bin_hist(mistic_handle_s* h, const uint32_t* bstart, uint32_t m, unsigned long long* hist) {
  MCK(cudaMemsetAsync(hist, 0, 32 * sizeof(unsigned long long), h->stream));
  const unsigned nb = std::max(1u, std::min((m + 255) / 256, 4u * (unsigned)h->sms));
  k_bin_hist<<<nb, 256, 0, h->stream>>>(bstart, m, hist);
  launched(h, "bin_hist");
}

void count_totals(mistic_handle_s* h, const uint32_t* nbr_cnt, const uint32_t* unit_cnt, const uint32_t* unit_cnt_tc,
                  uint32_t m, unsigned long long* tot) {
  MCK(cudaMemsetAsync(tot, 0, 3 * sizeof(unsigned long long), h->stream));
  const unsigned nb = std::max(1u, std::min((m + 255) / 256, 4u * (unsigned)h->sms));
  k_count_totals<<<nb, 256, 0, h->stream>>>(nbr_cnt, unit_cnt, unit_cnt_tc, m, tot);
  launched(h, "count_totals");
}

}  // namespace idx
}  // namespace mistic
