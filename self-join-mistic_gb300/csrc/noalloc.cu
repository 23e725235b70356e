// mistic_selfjoin_noalloc: an ε-self-join entry point that allocates no
// memory at all.
//
// Who needs it: callers that must not allocate device memory while they
// run.  Examples are a service whose device memory is entirely reserved up
// front by its own pool allocator (a fresh cudaMalloc can fail or fragment
// that pool), and a latency-critical path where the implicit device-wide
// synchronisation of cudaMalloc/cudaFree would stall every other stream of
// the process.  The regular entry point, mistic_selfjoin, grows and caches
// buffers in its handle, so it cannot serve them.
//
// How: the only scratch memory this path uses is the file-scope array
// `g_noalloc_scratch` below, a fixed MISTIC_NOALLOC_SCRATCH_BYTES block that
// every GPU loading the library holds until the process exits.  The caller
// passes the points and the pair buffer, both already on the device.  The
// join is a variant of the FP32-filter join kernel (join.cu) without the
// reference-point index: every pair i < j is a candidate, so it is meant for
// modest n (the scratch holds one FP32 copy of the points).
//
// Host code cannot use `g_noalloc_scratch` as an address: on the host that
// name is only a stand-in, and a kernel handed it would fault or, where the
// GPU can reach host memory, silently use the wrong memory.  So the first
// call on each device looks the device address up with cudaGetSymbolAddress
// (with that device current), checks the result and caches it; kernels get
// that pointer.  Under CUDA's default lazy module loading the array itself is only
// allocated when this module first loads on a device, i.e. at that first
// call: make it (a call with n = 0 does only the set-up) before a pool
// allocator reserves the device's memory.
//
// Inputs holding a NaN or an infinite coordinate are rejected with
// MISTIC_ERR_NOT_FINITE, as mistic_selfjoin does by default.
//
// Every call shares the one scratch block and it keeps the previous call's
// contents: each call clears the counters it relies on before use.  Calls
// whose work overlaps on the GPU (different streams or host threads at the
// same time) race on the scratch and must be serialised by the caller.
#include <math.h>
#include <string.h>

#include <algorithm>
#include <mutex>

#include "internal.cuh"

namespace mistic {
namespace {

constexpr size_t kScratchBytes = MISTIC_NOALLOC_SCRATCH_BYTES;
constexpr size_t kHeaderBytes = 256;  // counters, then the FP32 rows
constexpr int kThreads = 256;
constexpr int kCH = 32;      // home points per unit
constexpr uint32_t kSeg = 4096;  // candidate points per unit
constexpr int kMaxDevices = 64;

static __device__ __align__(256) unsigned char g_noalloc_scratch[kScratchBytes];

struct NaHeader {
  unsigned long long pairs;
  unsigned long long band;
  unsigned long long next_unit;
  unsigned long long r2max_bits;  // largest squared FP32 row norm, as FP64 bits
  unsigned long long nonfinite;   // non-zero: an input coordinate is NaN or infinite
};

struct NaParams {
  const void* raw;  // caller's rows (device)
  int raw_f32;
  uint32_t n, d, dpad;
  const float* xf;  // FP32 rows relative to row 0, in the scratch
  NaHeader* hdr;    // in the scratch
  float t_lo, t_hi;
  int all_fp64;     // 1: FP32 cannot separate the pairs; every candidate is decided in FP64
  double eps2;
  unsigned long long* pairs;  // caller's buffer, packed (i << 32 | j)
  unsigned long long cap;
  uint32_t nseg;
  unsigned long long n_units;
};

__device__ __forceinline__ double na_ld(const void* p, int f32, size_t i) {
  return f32 ? (double)((const float*)p)[i] : ((const double*)p)[i];
}

// FP32 copy of every row minus row 0 (zero padded to dpad), the largest
// squared row norm, and a flag for NaN or infinite input coordinates (one
// such value in row 0 would otherwise poison every FP32 row).
__global__ void k_na_convert(NaParams P) {
  const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
  double r2 = 0.0;
  bool bad = false;
  if (i < P.n) {
    float* row = const_cast<float*>(P.xf) + (size_t)i * P.dpad;
    for (uint32_t t = 0; t < P.dpad; ++t) {
      float v = 0.f;
      if (t < P.d) {
        const double xi = na_ld(P.raw, P.raw_f32, (size_t)i * P.d + t);
        bad |= !isfinite(xi);
        v = (float)(xi - na_ld(P.raw, P.raw_f32, t));
      }
      row[t] = v;
      r2 = fma((double)v, (double)v, r2);
    }
  }
  if (__any_sync(FULL_MASK, bad) && (threadIdx.x & 31) == 0) atomicExch(&P.hdr->nonfinite, 1ull);
#pragma unroll
  for (int o = 16; o; o >>= 1) r2 = fmax(r2, __shfl_xor_sync(FULL_MASK, r2, o));
  if ((threadIdx.x & 31) == 0 && r2 > 0.0)
    atomicMax(&P.hdr->r2max_bits, (unsigned long long)__double_as_longlong(r2));
}

__device__ __forceinline__ uint32_t na_scan(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// The reference predicate (src/utils.cu:296-309), no contraction.
__device__ __forceinline__ double na_exact(const NaParams& P, uint32_t i, uint32_t j) {
  double s = 0.0;
  for (uint32_t t = 0; t < P.d; ++t) {
    const double df = __dsub_rn(na_ld(P.raw, P.raw_f32, (size_t)i * P.d + t),
                                na_ld(P.raw, P.raw_f32, (size_t)j * P.d + t));
    s = __dadd_rn(s, __dmul_rn(df, df));
  }
  return s;
}

// Units: home chunk c (rows 32c .. 32c+31) against candidate segment s
// (rows s*kSeg .. s*kSeg+kSeg-1), candidates restricted to j > i.
__global__ void __launch_bounds__(kThreads) k_na_join(const NaParams P) {
  extern __shared__ float4 na_smem[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nq4 = P.dpad >> 2;
  float4* sA = na_smem + (size_t)w * kCH * nq4;
  const float4* X = (const float4*)P.xf;
  uint32_t band_cnt = 0;
  for (;;) {
    unsigned long long u = 0;
    if (lane == 0) u = atomicAdd(&P.hdr->next_unit, 1ull);
    u = __shfl_sync(FULL_MASK, u, 0);
    if (u >= P.n_units) break;
    const uint32_t c = (uint32_t)(u / P.nseg), s = (uint32_t)(u % P.nseg);
    const uint32_t a0 = c * kCH;
    const uint32_t na = min((uint32_t)kCH, P.n - a0);
    const uint32_t qlo = max(a0 + 1, s * kSeg), qhi = min(P.n, (s + 1) * kSeg);
    if (qlo >= qhi) continue;
    __syncwarp();
    for (uint32_t i = lane; i < kCH * nq4; i += 32)
      sA[i] = i < na * nq4 ? X[(size_t)a0 * nq4 + i] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    for (uint32_t qb = qlo; qb < qhi; qb += 32) {
      const uint32_t q = qb + lane;
      const bool qv = q < qhi;
      const float4* qrow = X + (size_t)(qv ? q : qlo) * nq4;
      float acc[kCH];
#pragma unroll
      for (int a = 0; a < kCH; ++a) acc[a] = 0.f;
      for (uint32_t cc = 0; cc < nq4; ++cc) {
        const float4 qq = qrow[cc];
#pragma unroll
        for (int a = 0; a < kCH; ++a) {
          const float4 aa = sA[a * nq4 + cc];
          float t;
          t = aa.x - qq.x; acc[a] = fmaf(t, t, acc[a]);
          t = aa.y - qq.y; acc[a] = fmaf(t, t, acc[a]);
          t = aa.z - qq.z; acc[a] = fmaf(t, t, acc[a]);
          t = aa.w - qq.w; acc[a] = fmaf(t, t, acc[a]);
        }
      }
      uint32_t m = 0, lo = 0;
      if (P.all_fp64) {
        // the FP32 values are not usable (an offset beyond FLT_MAX is inf and
        // inf - inf is NaN): every candidate goes to the FP64 decision
        m = FULL_MASK;
      } else {
#pragma unroll
        for (int a = 0; a < kCH; ++a) {
          m |= (acc[a] <= P.t_hi ? 1u : 0u) << a;
          lo |= (acc[a] <= P.t_lo ? 1u : 0u) << a;
        }
      }
      // valid home rows: a < na and a0 + a < q
      uint32_t valid = na >= 32 ? FULL_MASK : ((1u << na) - 1u);
      const int lim = (int)q - (int)a0;
      valid &= lim >= 32 ? FULL_MASK : (lim <= 0 ? 0u : ((1u << lim) - 1u));
      m = qv ? (m & valid) : 0u;
      if (!__any_sync(FULL_MASK, m != 0)) continue;
      uint32_t accm = lo & m, band = m & ~lo;
      while (band) {
        const int a = __ffs(band) - 1;
        band &= band - 1;
        ++band_cnt;
        if (na_exact(P, a0 + a, q) <= P.eps2) accm |= 1u << a;
      }
      const uint32_t cnt = __popc(accm);
      const uint32_t incl = na_scan(cnt);
      const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
      if (total == 0) continue;
      unsigned long long base = 0;
      if (lane == 31) base = atomicAdd(&P.hdr->pairs, (unsigned long long)total);
      base = __shfl_sync(FULL_MASK, base, 31);
      unsigned long long pos = base + incl - cnt;
      while (accm) {
        const int a = __ffs(accm) - 1;
        accm &= accm - 1;
        if (pos < P.cap) P.pairs[pos] = ((unsigned long long)(a0 + a) << 32) | q;
        ++pos;
      }
    }
  }
  const uint32_t tot = __shfl_sync(FULL_MASK, na_scan(band_cnt), 31);
  if (lane == 0 && tot) atomicAdd(&P.hdr->band, (unsigned long long)tot);
}

// Swap each packed (i << 32 | j) into memory order (i, j) as two uint32.
__global__ void k_na_to_ij(unsigned long long* p, unsigned long long n) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) p[i] = (p[i] >> 32) | (p[i] << 32);
}

std::mutex g_setup_mu;
void* g_scratch_dev[kMaxDevices] = {};

// Device address of the scratch array on the current device, looked up once
// per device with cudaGetSymbolAddress (the host-side symbol is not an
// address the GPU may use).
mistic_status scratch_address(void** out) {
  int dev = 0;
  if (cudaGetDevice(&dev) != cudaSuccess) {
    cudaGetLastError();
    return MISTIC_ERR_NO_DEVICE;
  }
  if (dev < 0 || dev >= kMaxDevices) return MISTIC_ERR_NO_DEVICE;
  std::lock_guard<std::mutex> lk(g_setup_mu);
  if (!g_scratch_dev[dev]) {
    void* p = nullptr;
    const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
    if (e != cudaSuccess || !p) {
      cudaGetLastError();
      return MISTIC_ERR_CUDA;
    }
    g_scratch_dev[dev] = p;
  }
  *out = g_scratch_dev[dev];
  return MISTIC_OK;
}

mistic_status cuda_status(cudaError_t e) {
  if (e == cudaSuccess) return MISTIC_OK;
  cudaGetLastError();
  return MISTIC_ERR_CUDA;
}

}  // namespace
}  // namespace mistic

extern "C" mistic_status mistic_selfjoin_noalloc(const void* d_pts, uint64_t n, uint32_t d, mistic_dtype dtype,
                                                 double eps, uint32_t* d_pairs, uint64_t pair_capacity,
                                                 uint64_t* pairs_ij, void* stream) {
  using namespace mistic;
  if (!pairs_ij) return MISTIC_ERR_INVALID_ARG;
  *pairs_ij = 0;
  if (dtype != MISTIC_F64 && dtype != MISTIC_F32) return MISTIC_ERR_INVALID_ARG;
  if (d == 0 || !(eps >= 0.0) || !std::isfinite(eps)) return MISTIC_ERR_INVALID_ARG;
  if (n > 0 && !d_pts) return MISTIC_ERR_INVALID_ARG;
  if (pair_capacity > 0 && !d_pairs) return MISTIC_ERR_INVALID_ARG;
  if ((uintptr_t)d_pairs % 8) return MISTIC_ERR_INVALID_ARG;
  const uint32_t dpad = (d + 3) & ~3u;
  if (d > MISTIC_NOALLOC_MAX_D || n >= 0xffffffffull ||
      (unsigned long long)n * dpad * sizeof(float) > kScratchBytes - kHeaderBytes)
    return MISTIC_ERR_TOO_LARGE;
  // set-up first, even for n < 2: a call with n = 0 only resolves the
  // scratch array on the current device (see the header)
  void* scratch = nullptr;
  mistic_status st = scratch_address(&scratch);
  if (st != MISTIC_OK) return st;
  if (n < 2) return MISTIC_OK;
  cudaStream_t s = (cudaStream_t)stream;
  NaParams P{};
  P.raw = d_pts;
  P.raw_f32 = dtype == MISTIC_F32;
  P.n = (uint32_t)n;
  P.d = d;
  P.dpad = dpad;
  P.hdr = (NaHeader*)scratch;
  P.xf = (const float*)((unsigned char*)scratch + kHeaderBytes);
  P.eps2 = eps * eps;
  P.pairs = (unsigned long long*)d_pairs;
  P.cap = pair_capacity;
  // the counters and the norm maximum must start at zero on every call
  if ((st = cuda_status(cudaMemsetAsync(P.hdr, 0, sizeof(NaHeader), s))) != MISTIC_OK) return st;
  k_na_convert<<<(unsigned)((n + kThreads - 1) / kThreads), kThreads, 0, s>>>(P);
  if ((st = cuda_status(cudaGetLastError())) != MISTIC_OK) return st;
  NaHeader hh{};
  if ((st = cuda_status(cudaMemcpyAsync(&hh, P.hdr, sizeof hh, cudaMemcpyDeviceToHost, s))) != MISTIC_OK) return st;
  if ((st = cuda_status(cudaStreamSynchronize(s))) != MISTIC_OK) return st;
  if (hh.nonfinite) return MISTIC_ERR_NOT_FINITE;
  double r2 = 0.0;
  memcpy(&r2, &hh.r2max_bits, sizeof r2);
  const double R = sqrt(r2) * (1.0 + 1e-12);
  const double eps2 = P.eps2;
  if (eps2 == 0.0 || eps2 < 1e-28 || !(R <= 1e15) || !filter_thresholds(d, eps2, R, &P.t_lo, &P.t_hi)) {
    P.t_lo = -1.0f;  // FP32 cannot separate these pairs: re-decide every candidate in FP64
    P.t_hi = INFINITY;
    P.all_fp64 = 1;
  }
  const uint32_t nchunks = (uint32_t)((n + kCH - 1) / kCH);
  P.nseg = (uint32_t)((n + kSeg - 1) / kSeg);
  P.n_units = (unsigned long long)nchunks * P.nseg;
  const size_t smem_warp = (size_t)kCH * dpad * sizeof(float);
  const int warps = (int)std::min<size_t>(kThreads / 32, std::max<size_t>(1, (160 * 1024) / smem_warp));
  const size_t smem = smem_warp * warps;
  if (smem > 48 * 1024 &&
      (st = cuda_status(cudaFuncSetAttribute(k_na_join, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                             (int)smem))) != MISTIC_OK)
    return st;
  int dev = 0, sms = 0, per_sm = 0;
  if ((st = cuda_status(cudaGetDevice(&dev))) != MISTIC_OK) return st;
  if ((st = cuda_status(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev))) != MISTIC_OK) return st;
  if ((st = cuda_status(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_na_join, warps * 32, smem))) !=
      MISTIC_OK)
    return st;
  if (per_sm < 1) return MISTIC_ERR_TOO_LARGE;
  const unsigned long long want = (P.n_units + warps - 1) / warps;
  const unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)per_sm * sms, want);
  k_na_join<<<grid, warps * 32, smem, s>>>(P);
  if ((st = cuda_status(cudaGetLastError())) != MISTIC_OK) return st;
  if ((st = cuda_status(cudaMemcpyAsync(&hh, P.hdr, sizeof hh, cudaMemcpyDeviceToHost, s))) != MISTIC_OK) return st;
  if ((st = cuda_status(cudaStreamSynchronize(s))) != MISTIC_OK) return st;
  const unsigned long long stored = std::min<unsigned long long>(hh.pairs, pair_capacity);
  if (stored) {
    k_na_to_ij<<<(unsigned)((stored + 255) / 256), 256, 0, s>>>(P.pairs, stored);
    if ((st = cuda_status(cudaGetLastError())) != MISTIC_OK) return st;
    if ((st = cuda_status(cudaStreamSynchronize(s))) != MISTIC_OK) return st;
  }
  *pairs_ij = hh.pairs;
  return hh.pairs > pair_capacity ? MISTIC_ERR_PAIR_OVERFLOW : MISTIC_OK;
}
