// C ABI and pipeline orchestration of the ε-self-join (include/mistic.h).
//
// Reference counterpart: nodeLauncher5, src/launcher.cu:3093-3532, which
// builds the node net on the host (buildNodeNet, src/nodes.cu:5-356),
// flattens it into CSR arrays, plans batches, copies everything to the
// device, and per batch launches nodeByPoint5, copies the pair count back,
// sorts the pairs and rebuilds a host neighbour table.  Here every stage runs
// on the device on one stream of the handle:
//
//   colstats -> (sample covariance) -> reference points (host, small)
//   -> FP64 RP distances -> packed bin keys -> radix sort -> bin starts
//   -> sorted-order gather -> ±1 neighbour enumeration (count, scan, fill)
//   -> persistent join with pair compaction -> (pair sort) -> read-back
//
// The host synchronises only for a handful of scalars (key layout, bin and
// work-list sizes, final counts).
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include <algorithm>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <fstream>
#include <map>
#include <atomic>
#include <mutex>
#include <thread>
#include <functional>
#include <unordered_map>
#include <vector>

#include <sys/stat.h>

#include "internal.cuh"

namespace mistic {

void pairs_to_ij(mistic_handle_s* h, unsigned long long* p, size_t n);
void csr_edges(mistic_handle_s* h, const unsigned long long* pairs, size_t np, size_t n, unsigned long long* e);
void csr_split(mistic_handle_s* h, const unsigned long long* e, size_t E, uint32_t* nbrs, unsigned long long* offs,
               size_t n);

// ------------------------------------------------------------------ plumbing

void throw_cuda(cudaError_t e, const char* what, const char* file, int line) {
  char buf[512];
  snprintf(buf, sizeof buf, "%s failed: %s (%s:%d)", what, cudaGetErrorString(e), file, line);
  if (e == cudaErrorMemoryAllocation) {
    cudaGetLastError();
    throw Error(MISTIC_ERR_OUT_OF_MEMORY, buf);
  }
  throw Error(MISTIC_ERR_CUDA, buf);
}

void launched(mistic_handle_s* h, const char* what) {
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) throw_cuda(e, what, __FILE__, __LINE__);
  ++h->launches;
}

void* Arena::get(const std::string& name, size_t bytes) {
  if (bytes == 0) bytes = 16;
  Buf& b = bufs[name];
  if (b.bytes < bytes) {
    if (b.p) {
      if (stream) MCK(cudaStreamSynchronize(stream));
      MCK(cudaFree(b.p));
    }
    b.p = nullptr;
    b.bytes = 0;
    size_t want = bytes + bytes / 8;  // head-room against regrowth
    cudaError_t e = cudaMalloc(&b.p, want);
    if (e != cudaSuccess) {
      cudaGetLastError();
      e = cudaMalloc(&b.p, bytes);
      want = bytes;
    }
    if (e != cudaSuccess) throw_cuda(e, ("cudaMalloc " + name).c_str(), __FILE__, __LINE__);
    b.bytes = want;
  }
  return b.p;
}

void Arena::release_all() {
  for (auto& kv : bufs)
    if (kv.second.p) cudaFree(kv.second.p);
  bufs.clear();
}

// Threshold pair for the FP32 filter.  With x~ = fl32(x - c), t~ =
// fl32(x~ - y~), s32 the FP32 fma sum of t~^2, D the exact distance, R the
// largest ||x~||, u = 2^-24 (inflated for the FP64 centring), the error is
//   |s32 - D^2| <= E(D) = (1+g_d)(2u(2R+D)D + u^2(2R+D)^2) + g_d D^2 + tiny,
// g_d = d u / (1 - d u).  The reference value s64 (sequential FP64) obeys
// |s64 - D^2| <= g64 D^2.  With D' = 1.1 sqrt(eps2) and E' = E(D'), every
// pair with s32 <= T_lo = eps2/(1+g64) - E' has s64 <= eps2, and every pair
// with s32 > T_hi = eps2/(1-g64) + E' has s64 > eps2: for D <= D' directly,
// and for D > D' because D^2 - E(D) grows with D and already exceeds T_hi at
// D' whenever E' <= 0.1 eps2.  Returns false when that condition fails (the
// coordinates are too large relative to ε for FP32); the caller then joins
// in FP64.
bool filter_thresholds(uint32_t d, double eps2, double R, float* t_lo, float* t_hi) {
  const double u = ldexp(1.0, -24) * (1.0 + ldexp(1.0, -20));
  const double gd = d * u / (1.0 - d * u);
  const double g64 = (d + 2) * ldexp(1.0, -53) * 1.01;
  const double Dp = 1.1 * sqrt(eps2);
  const double tiny = (double)(d + 2) * ldexp(1.0, -126);
  const double E = (1.0 + gd) * (2.0 * u * (2.0 * R + Dp) * Dp + u * u * (2.0 * R + Dp) * (2.0 * R + Dp)) +
                   gd * Dp * Dp + tiny;
  if (!(E <= 0.1 * eps2)) return false;
  double lo = eps2 / (1.0 + g64) - E;
  double hi = eps2 / (1.0 - g64) + E;
  lo *= 1.0 - 1e-12;
  hi *= 1.0 + 1e-12;
  float flo = lo > 0 ? (float)lo : -1.0f;
  if ((double)flo > lo) flo = nextafterf(flo, -INFINITY);
  float fhi = (float)hi;
  if ((double)fhi < hi) fhi = nextafterf(fhi, INFINITY);
  *t_lo = flo;
  *t_hi = fhi;
  return true;
}

void allow_max_dyn_smem_impl(const void* kern) {
  static std::mutex mu;
  static std::map<const void*, cudaError_t>* done = new std::map<const void*, cudaError_t>;
  std::lock_guard<std::mutex> g(mu);
  auto it = done->find(kern);
  if (it == done->end()) {
    cudaError_t err = cudaSuccess;
    int dev = 0, optin = 0;
    cudaFuncAttributes fa{};
    if ((err = cudaGetDevice(&dev)) == cudaSuccess &&
        (err = cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev)) == cudaSuccess &&
        (err = cudaFuncGetAttributes(&fa, kern)) == cudaSuccess &&
        (err = cudaFuncSetAttribute(kern, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                    optin - (int)fa.sharedSizeBytes)) == cudaSuccess)
      err = cudaFuncSetAttribute(kern, cudaFuncAttributePreferredSharedMemoryCarveout, 100);
    it = done->emplace(kern, err).first;
  }
  MCK(it->second);
}

namespace {

// Process-wide cache of pinned host blocks for result arrays: a device-to-
// host copy into pinned memory runs at the link's speed, one into fresh
// pageable memory stalls on page faults.  Blocks come in size classes of at
// most 12.5% waste, are handed to a result and come back here from
// mistic_result_free; up to kMaxCached bytes stay cached for the next call.
class PinnedCache {
 public:
  void* acquire(size_t bytes) {
    const size_t cls = size_class(bytes);
    {
      std::lock_guard<std::mutex> g(mu_);
      auto it = free_.lower_bound(cls);
      if (it != free_.end() && it->first <= 2 * cls) {
        void* p = it->second;
        cached_ -= it->first;
        free_.erase(it);
        return p;
      }
    }
    void* p = nullptr;
    if (cudaHostAlloc(&p, cls, cudaHostAllocPortable) != cudaSuccess) {
      cudaGetLastError();  // clear; the caller falls back to pageable memory
      return nullptr;
    }
    std::lock_guard<std::mutex> g(mu_);
    size_[p] = cls;
    return p;
  }
  // false: not a block of this cache
  bool release(void* p) {
    size_t sz = 0;
    {
      std::lock_guard<std::mutex> g(mu_);
      auto it = size_.find(p);
      if (it == size_.end()) return false;
      sz = it->second;
      if (cached_ + sz <= kMaxCached) {
        free_.emplace(sz, p);
        cached_ += sz;
        return true;
      }
      size_.erase(it);
    }
    cudaFreeHost(p);
    return true;
  }

 private:
  static constexpr size_t kMaxCached = 12ull << 30;
  static size_t size_class(size_t bytes) {
    if (bytes <= (1u << 16)) return 1u << 16;
    int lg = 63 - __builtin_clzll((unsigned long long)bytes);
    const size_t step = (size_t)1 << (lg - 3);
    return (bytes + step - 1) / step * step;
  }
  std::mutex mu_;
  std::multimap<size_t, void*> free_;
  std::unordered_map<void*, size_t> size_;
  size_t cached_ = 0;
};

PinnedCache& pinned_cache() {
  static PinnedCache* c = new PinnedCache;  // never destroyed: blocks may outlive static teardown
  return *c;
}

// A pinned block owned by a call until it is handed to the result.  Kernels
// of the call's stream may write it (host pair lists): before it goes back
// to the cache -- a larger one replacing it, or an error unwinding the call --
// the stream is drained.
struct PinnedHold {
  void* p = nullptr;
  cudaStream_t stream = nullptr;
  void reset() {
    if (p) {
      cudaStreamSynchronize(stream);
      cudaGetLastError();
      pinned_cache().release(p);
    }
    p = nullptr;
  }
  ~PinnedHold() { reset(); }
};

template <class T>
T* abuf(mistic_handle_s* h, const char* name, size_t count) {
  return (T*)h->arena.get(name, count * sizeof(T));
}

void d2h(mistic_handle_s* h, void* dst, const void* src, size_t bytes) {
  MCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyDeviceToHost, h->stream));
  MCK(cudaStreamSynchronize(h->stream));
}

// Host -> device copy of a caller's (pageable) array, stream-ordered on the
// handle's stream.  Small copies go straight to cudaMemcpyAsync.  Large ones
// go through the handle's pinned staging ring: kStageThreads host threads
// each copy every kStageThreads-th chunk into one of their two slots and
// issue that slot's DMA, so the host-side copies run in parallel and overlap
// the DMAs (a pageable cudaMemcpyAsync is one driver-staged copy at a time,
// measured at 7.3 GB/s for the 720 MB input of the 5M x 18 join).  The
// ring (128 MB pinned) is allocated at the handle's first large copy.  A slot is
// refilled only after the event recorded behind its previous DMA has
// completed.  The call returns once every DMA has been issued; the source
// may be reused by the caller after the stream has passed them.
constexpr size_t kStageSlotBytes = 8u << 20;
constexpr int kStageThreads = 8;
constexpr int kStageSlots = 2 * kStageThreads;
constexpr size_t kStageMin = 128u << 20;
// below this a plain copy costs about what a kernel launch does
constexpr size_t kHostReadMin = 64u << 10;
static_assert(kStageSlots <= (int)(sizeof(((mistic_handle_s*)nullptr)->stage_ev) / sizeof(cudaEvent_t)),
              "one event per staging slot");

// Grid-stride copy of n16 16-byte chunks from host memory the GPU can
// address directly (pageable memory through the host page tables).
__global__ void k_copy_from_host(const uint4* __restrict__ src, uint4* __restrict__ dst, size_t n16) {
  for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n16; i += (size_t)gridDim.x * blockDim.x)
    dst[i] = src[i];
}

// Host rows to the device.  Where the GPU reads pageable host memory itself
// (GB300 with a Grace host: coherent NVLink-C2C and the host's page tables),
// one kernel pulls the caller's array straight into HBM: 720 MB in 3.8 ms,
// the link's rate, against 9 ms through the staging ring below, which pays
// a host memcpy into pinned slots.  The kernel also serves inputs down to
// 64 KB, which a plain pageable copy moves at a few GB/s (the instances of a
// batch).  Elsewhere inputs of 128 MB or more go through that ring, smaller
// ones through one plain copy.
void h2d(mistic_handle_s* h, void* dst, const void* src, size_t bytes) {
  bool kernel = bytes >= kHostReadMin && h->host_reads && (uintptr_t)src % 16 == 0 && (uintptr_t)dst % 16 == 0;
  bool timed = false;
  if (kernel && bytes >= kStageMin) {
    // The kernel usually reads at the link's rate (about 200 GB/s), but on
    // some machines and in some processes the same copy ran at 20-40 GB/s
    // (by every sign bound by the GPU's translations of the caller's pages),
    // below the staging ring's ~80 GB/s, which a host-side memcpy feeds.
    // After such a copy the next 8 large ones take the ring, then the kernel
    // is tried again.
    if (h->hr_bytes) {
      float ms = 0.f;
      if (cudaEventElapsedTime(&ms, h->hr_ev[0], h->hr_ev[1]) == cudaSuccess && ms > 0.f &&
          (double)h->hr_bytes / (ms * 1e6) < 70.0)
        h->hr_skip = 8;
      cudaGetLastError();
      h->hr_bytes = 0;
    }
    if (h->hr_skip) {
      --h->hr_skip;
      kernel = false;
    } else {
      for (auto& e : h->hr_ev)
        if (!e && cudaEventCreate(&e) != cudaSuccess) e = nullptr;
      cudaGetLastError();
      timed = h->hr_ev[0] && h->hr_ev[1];
    }
  }
  if (kernel) {
    const size_t n16 = bytes / 16;
    const unsigned grid = (unsigned)std::min<size_t>((size_t)h->sms * 8, (n16 + 255) / 256);
    if (timed) MCK(cudaEventRecord(h->hr_ev[0], h->stream));
    k_copy_from_host<<<grid, 256, 0, h->stream>>>(static_cast<const uint4*>(src), static_cast<uint4*>(dst), n16);
    launched(h, "copy_from_host");
    if (timed) {
      MCK(cudaEventRecord(h->hr_ev[1], h->stream));
      h->hr_bytes = bytes;
    }
    if (bytes % 16)
      MCK(cudaMemcpyAsync(static_cast<unsigned char*>(dst) + n16 * 16, static_cast<const unsigned char*>(src) + n16 * 16,
                          bytes % 16, cudaMemcpyHostToDevice, h->stream));
    return;
  }
  if (bytes >= kStageMin && !h->stage) {
    void* p = nullptr;
    if (cudaHostAlloc(&p, kStageSlots * kStageSlotBytes, cudaHostAllocPortable) == cudaSuccess) {
      bool ok = true;
      for (int i = 0; i < kStageSlots && ok; ++i)
        ok = cudaEventCreateWithFlags(&h->stage_ev[i], cudaEventDisableTiming) == cudaSuccess;
      if (ok) {
        h->stage = p;
      } else {
        for (auto& e : h->stage_ev)
          if (e) cudaEventDestroy(e), e = nullptr;
        cudaFreeHost(p);
      }
    }
    cudaGetLastError();  // no staging ring: the plain copy below
  }
  if (bytes < kStageMin || !h->stage) {
    MCK(cudaMemcpyAsync(dst, src, bytes, cudaMemcpyHostToDevice, h->stream));
    return;
  }
  const size_t nchunks = (bytes + kStageSlotBytes - 1) / kStageSlotBytes;
  std::atomic<int> err{(int)cudaSuccess};
  auto worker = [&](int t) {
    cudaSetDevice(h->device);
    uint32_t use = 0;
    for (size_t c = (size_t)t; c < nchunks && err.load() == (int)cudaSuccess; c += kStageThreads, ++use) {
      const int slot = t + kStageThreads * (int)(use & 1);
      unsigned char* sb = static_cast<unsigned char*>(h->stage) + (size_t)slot * kStageSlotBytes;
      const size_t off = c * kStageSlotBytes, len = std::min(kStageSlotBytes, bytes - off);
      cudaError_t e = cudaEventSynchronize(h->stage_ev[slot]);  // the slot's previous DMA is done
      if (e == cudaSuccess) {
        memcpy(sb, static_cast<const unsigned char*>(src) + off, len);
        e = cudaMemcpyAsync(static_cast<unsigned char*>(dst) + off, sb, len, cudaMemcpyHostToDevice, h->stream);
      }
      if (e == cudaSuccess) e = cudaEventRecord(h->stage_ev[slot], h->stream);
      if (e != cudaSuccess) {
        int ok = (int)cudaSuccess;
        err.compare_exchange_strong(ok, (int)e);
      }
    }
  };
  std::vector<std::thread> pool;
  const int nt = (int)std::min<size_t>(kStageThreads, nchunks);
  for (int t = 1; t < nt; ++t) pool.emplace_back(worker, t);
  worker(0);
  for (auto& th : pool) th.join();
  MCK((cudaError_t)err.load());
}

struct PhaseClock {
  mistic_handle_s* h;
  bool on;
  int n = 0;
  void mark() {
    if (on && n < 16) MCK(cudaEventRecord(h->ev[n++], h->stream));
  }
  double ms(int a, int b) {
    if (!on || b >= n || a >= n) return 0.0;
    float v = 0;
    MCK(cudaEventElapsedTime(&v, h->ev[a], h->ev[b]));
    return v;
  }
};

int bit_length(uint64_t v) {
  int b = 0;
  while (v) {
    ++b;
    v >>= 1;
  }
  return b;
}

// Smallest home bin joined on the tensor cores (MISTIC_TC_MIN_BIN overrides
// it, for tuning).  A tensor-core tile costs about the same per candidate row
// whatever its number of home rows, a CUDA-core unit costs d FMAs per cell,
// so small bins go to the CUDA cores.  Measured on GB300 (whole join, ms):
//   5M x 18:    T = 48: 150.2, 61: 147.0, 80: 145.2, 100: 145.1, 128: 146.8
//   515k x 90:  T = 1: 259.9, 2: 261.9, 4: 261.9, 8: 263.3
// hence 29000 / d^2, clamped to [1, 96].
uint32_t tc_min_bin(uint32_t d, bool wide) {
  const char* e = getenv("MISTIC_TC_MIN_BIN");
  if (e && *e) return (uint32_t)std::max(1l, strtol(e, nullptr, 10));
  // long rows (K-chunked kernel): every bin.  Even a one-row bin is joined
  // faster on the tensor cores (a 128-row tile at ~1/128 use) than by the
  // FP32 CUDA-core kernel, whose units of a small home bin against a very
  // large neighbour bin (one segment holds a whole bin) run on single warps:
  // on the 5M x 384 workload such units took 2.1 s of a 14 s join at T = 8.
  if (wide) return 1;
  return (uint32_t)std::min(96.0, std::max(1.0, std::floor(29000.0 / ((double)d * d))));
}

// Relative error allowance per (|a'| + |q'|)^2 + 1.2 eps2 of a tensor-core
// join (TcParams.kappa): operand rounding per |a_k||q_k| + FP32
// accumulation (2^-19 per MMA instruction along K; measured worst case on
// GB300 below 0.09 of that) + FP32 norms + ...  Operand rounding: bf16 keeps
// 8 significant bits (unit roundoff 2^-8) and tf32 11 (2^-11), so with
// x = hi + lo + r, |x - hi| <= 2^-8 |x|, |r| <= 2^-16 |x|:
//   split bf16 (hi.hi + hi.lo + lo.hi)  3.02 * 2^-16,
//   single bf16                         2 * 2^-8 + 2^-16 = 2^-7 + 2^-16,
//   tf32 (rounded to nearest)           2 * 2^-11 + 2^-22 = 2^-10 + 2^-22,
// and then
// FP32 norms + the rounding of the folded column |q'|^2 - T (short rows), or
// of the three FP32 operations forming D' = |a|^2 - 2G + (|q|^2 - T) in the
// long-row kernel's epilogue (each within u (|a| + |q|)^2 + u T).
double tc_kappa(uint32_t d, bool wide, int prec) {
  const double u = ldexp(1.0, -24) * (1.0 + ldexp(1.0, -20));
  const double gd = d * u / (1.0 - d * u);
  const double op = prec == 1 ? ldexp(1.0, -7) + ldexp(1.0, -16)
                              : (prec == 2 ? ldexp(1.0, -10) + ldexp(1.0, -22) : 3.02 * ldexp(1.0, -16));
  const int n_mma = wide ? (prec == 0 ? 3 : 1) * (int)join::tcw_kd(d, prec) / (prec == 2 ? 8 : 16)
                         : 3 * join::tc_kp(d) / 16;
  return ((op + n_mma * 1.01 * ldexp(1.0, -19)) * (1.0 + gd) + gd + (wide ? 5.0 : 1.0) * u) * 1.01;
}

// Operand precision of the K-chunked tensor-core join.  TF32 mode: tf32.
// Otherwise single bf16 (a third of the split's tensor work) when even the
// widest column's bound -- rows at the largest norm R from the centre --
// stays within the cap of eps^2 / 10 (no column is left wholly to FP64);
// else split bf16.  MISTIC_TC_PREC=split|bf16 overrides (tuning).
int tc_precision(mistic_mode mode, uint32_t d, double eps2, double R) {
  if (mode == MISTIC_MODE_TF32) return 2;
  if (const char* e = getenv("MISTIC_TC_PREC")) {
    if (!strcmp(e, "split")) return 0;
    if (!strcmp(e, "bf16")) return 1;
  }
  const double u = ldexp(1.0, -24);
  const double rs = 2.0 * R, Dp = 1.1 * sqrt(eps2);
  const double delta = 2.0 * u * R + u * rs;
  const double E = tc_kappa(d, true, 1) * (rs * rs + 1.2 * eps2) + delta * (2.0 * Dp + delta);
  return E <= 0.1 * eps2 ? 1 : 0;
}

// Rows of 32 < d <= 126 on the K-chunked kernel too, when its globally
// centred bound keeps the band narrow: split-bf16 error for the widest
// columns (rows at the largest norm R) at most eps^2 / 100.  The short-row
// kernel centres each unit on its first row, which keeps the bound small
// whatever the coordinates, but converts every candidate tile on its CUDA
// cores; the K-chunked kernel reads rows prepared once.  On the 515k x 90
// workload (eps^2 = 50, R ~ 15) the short-row kernel was latency-bound on
// that conversion (issue 28 %, tensor pipe 14 %, 237 ms).  MISTIC_TC_WIDE=0/1
// overrides.
bool tcw_for_medium_rows(uint32_t d, double eps2, double R) {
  if (const char* e = getenv("MISTIC_TC_WIDE")) return *e == '1';
  if (d <= 32) return false;
  const double u = ldexp(1.0, -24);
  const double rs = 2.0 * R, Dp = 1.1 * sqrt(eps2);
  const double delta = 2.0 * u * R + u * rs;
  const double E = tc_kappa(d, true, 0) * (rs * rs + 1.2 * eps2) + delta * (2.0 * Dp + delta);
  return E <= 0.01 * eps2;
}

void check_handle(mistic_handle h) {
  if (!h) throw Error(MISTIC_ERR_INVALID_ARG, "null handle");
  MCK(cudaSetDevice(h->device));
}

// ------------------------------------------------------------------ autotuner
// The reference fixes its launch shape at compile time (include/params.cuh:
// 20-87: TPP, ILP, KB, BS, CALC_PER_BATCH) and its batch plan by a formula
// (src/launcher.cu:3202-3249).  Here the tensor-core join's two free choices
// -- the smallest home bin it takes (smaller bins go to the CUDA-core join)
// and, for the K-chunked kernel, split or single bf16 operands -- are timed
// on a fixed sample of the actual work (mistic_opts.home_sample) the first
// time a shape is seen, and cached.  Shape key: d, dtype, kernel, the
// point-weighted bin-size histogram (classes of the median and the 90th
// percentile point's bin), and log2(R^2 / eps^2) (how wide the band is
// against the rows' norms).  Cache: in memory, and lines of
// "key <TAB> tc_min <TAB> precision <TAB> ms" in MISTIC_TUNE_CACHE (default
// $HOME/.cache/mistic/tune.tsv), read once per process.
struct TuneCandidate {
  uint32_t tc_min;
  int prec;
};
struct Tuned {
  uint32_t tc_min = 0;
  int prec = 0;
};

class TuneCache {
 public:
  bool find(const std::string& key, Tuned* t) {
    std::lock_guard<std::mutex> g(mu_);
    load();
    auto it = map_.find(key);
    if (it == map_.end()) return false;
    *t = it->second;
    return true;
  }
  void put(const std::string& key, const Tuned& t, double ms) {
    std::lock_guard<std::mutex> g(mu_);
    load();
    map_[key] = t;
    const std::string path = file();
    if (path.empty()) return;
    const size_t slash = path.rfind('/');
    if (slash != std::string::npos && slash > 0) {  // create the directory (one level and its parent)
      const std::string dir = path.substr(0, slash);
      const size_t s2 = dir.rfind('/');
      if (s2 != std::string::npos && s2 > 0) mkdir(dir.substr(0, s2).c_str(), 0755);
      mkdir(dir.c_str(), 0755);
    }
    std::ofstream f(path, std::ios::app);
    if (f) f << key << '\t' << t.tc_min << '\t' << t.prec << '\t' << ms << '\n';
  }

 private:
  static std::string file() {
    if (const char* e = getenv("MISTIC_TUNE_CACHE")) return std::string(e);
    if (const char* hm = getenv("HOME")) return std::string(hm) + "/.cache/mistic/tune.tsv";
    return std::string();
  }
  void load() {
    if (loaded_) return;
    loaded_ = true;
    const std::string path = file();
    if (path.empty()) return;
    std::ifstream f(path);
    std::string line;
    while (std::getline(f, line)) {
      const size_t a = line.find('\t');
      if (a == std::string::npos) continue;
      const size_t b = line.find('\t', a + 1);
      if (b == std::string::npos) continue;
      Tuned t;
      t.tc_min = (uint32_t)strtoul(line.c_str() + a + 1, nullptr, 10);
      t.prec = atoi(line.c_str() + b + 1);
      if (t.tc_min >= 1 && t.prec >= 0 && t.prec <= 1) map_[line.substr(0, a)] = t;  // later lines win
    }
  }
  std::mutex mu_;
  bool loaded_ = false;
  std::map<std::string, Tuned> map_;
};

TuneCache& tune_cache() {
  static TuneCache* c = new TuneCache;
  return *c;
}

// times one candidate on the home-point sample 1/sample; reports the sample's
// candidate pairs and work units
using TuneMeasure = std::function<void(const TuneCandidate&, uint32_t sample, double* ms, unsigned long long* cands,
                                       unsigned long long* units)>;

// Looks the shape up, or times the candidates on a sample and records the
// fastest.  Returns false when tuning is off (the defaults then stand).
bool tune_lookup(mistic_handle_s* h, const mistic_opts& o, uint32_t d, mistic_dtype dt, bool wide, int prec_default,
                 const uint32_t* bstart, uint32_t m, double eps2, double R, Tuned* out,
                 const TuneMeasure& measure) {
  int want = o.autotune;
  if (const char* e = getenv("MISTIC_AUTOTUNE")) want = atoi(e) > 0 ? 1 : (atoi(e) < 0 || *e == '0' ? -1 : want);
  if (want < 0) return false;
  unsigned long long* hist_d = abuf<unsigned long long>(h, "tune_hist", 32);
  idx::bin_hist(h, bstart, m, hist_d);
  unsigned long long hist[32];
  d2h(h, hist, hist_d, sizeof hist);
  unsigned long long tot = 0;
  for (int i = 0; i < 32; ++i) tot += hist[i];
  if (want == 0 && tot < 1000000ull) return false;  // small joins: the defaults, no tuning cost
  int c50 = 0, c90 = 0;
  {
    unsigned long long acc = 0;
    bool got50 = false;
    for (int i = 0; i < 32; ++i) {
      acc += hist[i];
      if (!got50 && 2 * acc >= tot) c50 = i, got50 = true;
      if (10 * acc >= 9 * tot) {
        c90 = i;
        break;
      }
    }
  }
  const int eps_cls = (eps2 > 0 && R > 0) ? (int)std::floor(std::log2(R * R / eps2)) : 0;
  char key[160];
  snprintf(key, sizeof key, "v4 d=%u dt=%d %s bins=%d,%d r2e=%d", d, (int)dt, wide ? "tcw" : "tc", c50, c90, eps_cls);
  if (tune_cache().find(key, out)) return true;
  // candidates
  std::vector<TuneCandidate> cands;
  if (wide) {
    std::vector<int> precs = {0};
    if (prec_default == 1) precs.push_back(1);  // single bf16 only where its bound fits the cap
    for (int pr : precs) cands.push_back({1u, pr});  // every bin on the tensor cores (see tc_min_bin)
  } else {
    const uint32_t t0 = tc_min_bin(d, false);
    for (uint32_t t : {std::max(1u, t0 / 2), std::max(1u, 3 * t0 / 4), t0, std::min(512u, 3 * t0 / 2),
                       std::min(512u, 2 * t0)})
      if (cands.empty() || cands.back().tc_min != t) cands.push_back({t, 0});
  }
  // sample: about 1/64 of the home points, but enough work units that the
  // persistent grid is not timed on its tail (units of long rows are few and
  // large: at least ~20 a CTA), and no more than a few hundred ms a run
  uint32_t S = 64;
  double best = 1e300;
  Tuned bt{cands[0].tc_min, cands[0].prec};
  const unsigned long long want_units = 20ull * (unsigned long long)h->sms;
  // two rounds, the second in reverse order, each candidate keeping its
  // faster run: neighbouring thresholds differ by a few percent, about what
  // one run of a sample varies
  std::vector<double> t_best(cands.size(), 1e300);
  for (int round = 0; round < 2; ++round) {
    for (size_t j = 0; j < cands.size(); ++j) {
      const size_t i = round == 0 ? j : cands.size() - 1 - j;
      double ms = 0;
      unsigned long long cc = 0, uu = 0;
      measure(cands[i], S, &ms, &cc, &uu);
      if (round == 0 && i == 0) {
        uint32_t S2 = S;
        if (uu < want_units) S2 = (uint32_t)std::max(1.0, S * (double)uu / (double)want_units);
        if (ms * S / S2 > 400.0) S2 = (uint32_t)std::min(4096.0, std::ceil(S * ms / 400.0));
        if (S2 != S) {
          S = S2;
          measure(cands[i], S, &ms, &cc, &uu);
        }
      }
      if (getenv("MISTIC_DEBUG"))
        fprintf(stderr, "[mistic] tune %s: tc_min=%u prec=%d sample 1/%u: %.3f ms (%llu candidates)\n", key,
                cands[i].tc_min, cands[i].prec, S, ms, cc);
      t_best[i] = std::min(t_best[i], ms);
    }
  }
  for (size_t i = 0; i < cands.size(); ++i)
    if (t_best[i] < best) {
      best = t_best[i];
      bt = Tuned{cands[i].tc_min, cands[i].prec};
    }
  tune_cache().put(key, bt, best);
  *out = bt;
  return true;
}

// ------------------------------------------------------------------ the pipeline

// Phase one of a fused batch join (mistic_batch_selfjoin): run_selfjoin
// builds the instance's index and work lists, and then -- when the instance
// joins on the FP32 filter and/or the short-row tensor-core kernel --
// copies them into device memory obtained from `alloc` and describes them
// here instead of joining.  Ids are shifted by row0 so that pairs of
// different instances stay apart.  Instances that need the plain FP64 join
// or the K-chunked kernel are joined in full as usual (exported = false).
struct BatchExport {
  uint32_t row0 = 0;
  std::function<void*(size_t)> alloc;  // device bytes (256-byte aligned), or null when the batch arena is full
  bool exported = false;
  InstDesc desc{};
  uint32_t dpad32 = 0;
  const Unit* units = nullptr;     // CUDA-core units, in the allocated memory
  uint32_t n_units = 0;
  const Unit* units_tc = nullptr;  // tensor-core units
  uint32_t n_units_tc = 0;
  int CH = 0;                      // CUDA-core chunk
};

// Pair ring drain: the entries [0, m) that hold a pair of a unit not
// deferred in this pass, compacted into out (one atomic per warp).
__global__ void k_ring_drain(const unsigned long long* __restrict__ ring, const uint32_t* __restrict__ tags,
                             const uint32_t* __restrict__ deferred, unsigned long long m,
                             unsigned long long* __restrict__ out, unsigned long long* __restrict__ out_n) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  bool keep = false;
  unsigned long long v = 0;
  if (i < m) {
    const uint32_t t = tags[i];
    keep = t != 0xffffffffu && !deferred[t];
    if (keep) v = ring[i];
  }
  const uint32_t b = __ballot_sync(0xffffffffu, keep);
  if (!b) return;
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == 0) base = atomicAdd(out_n, (unsigned long long)__popc(b));
  base = __shfl_sync(0xffffffffu, base, 0);
  if (keep) out[base + __popc(b & ((1u << lane) - 1u))] = v;
}

// Clears the deferred flags of the tags in list[0 .. n).
__global__ void k_clear_flags(uint32_t* __restrict__ flags, const uint32_t* __restrict__ list, unsigned long long n) {
  const unsigned long long i = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) flags[list[i]] = 0u;
}

// inv[ids[p]] = p: sorted position of every original row id.
__global__ void k_inverse_perm(const uint32_t* __restrict__ ids, size_t n, uint32_t* __restrict__ inv) {
  const size_t p = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (p < n) inv[ids[p]] = (uint32_t)p;
}

__global__ void k_add_u32(const uint32_t* __restrict__ src, uint32_t* __restrict__ dst, size_t n, uint32_t add) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) dst[i] = src[i] + add;
}

void run_selfjoin(mistic_handle h, const void* pts, uint64_t n, uint32_t d, mistic_dtype dt, uint32_t k,
                  double eps, const mistic_opts* opts_in, mistic_result* r, BatchExport* ex = nullptr) {
  const auto wall0 = std::chrono::steady_clock::now();
  mistic_opts o;
  mistic_opts_init(&o);
  if (opts_in) {
    if (opts_in->struct_size != sizeof(mistic_opts))
      throw Error(MISTIC_ERR_INVALID_ARG, "mistic_opts.struct_size mismatch (call mistic_opts_init)");
    o = *opts_in;
  }
  if (!r) throw Error(MISTIC_ERR_INVALID_ARG, "null result");
  memset(r, 0, sizeof(*r));
  check_handle(h);
  if (dt != MISTIC_F64 && dt != MISTIC_F32) throw Error(MISTIC_ERR_INVALID_ARG, "unknown dtype");
  if (d == 0) throw Error(MISTIC_ERR_INVALID_ARG, "d must be >= 1");
  if (d > MAX_D) throw Error(MISTIC_ERR_TOO_LARGE, "d above the supported maximum (4096)");
  if (!(eps >= 0.0) || !std::isfinite(eps)) throw Error(MISTIC_ERR_INVALID_ARG, "eps must be finite and >= 0");
  if (k > MAX_K) throw Error(MISTIC_ERR_INVALID_ARG, "k above the supported maximum (16)");
  if (n >= 0xffffffffull) throw Error(MISTIC_ERR_TOO_LARGE, "n must be below 2^32 - 1");
  if (n > 0 && !pts) throw Error(MISTIC_ERR_INVALID_ARG, "null points");
  if (o.mode != MISTIC_MODE_AUTO && o.mode != MISTIC_MODE_FP64 && o.mode != MISTIC_MODE_FP32 &&
      o.mode != MISTIC_MODE_BF16 && o.mode != MISTIC_MODE_TF32)
    throw Error(MISTIC_ERR_INVALID_ARG, "unknown mode");
  if (o.pairs != MISTIC_PAIRS_NONE && o.pairs != MISTIC_PAIRS_HOST && o.pairs != MISTIC_PAIRS_DEVICE)
    throw Error(MISTIC_ERR_INVALID_ARG, "unknown pairs destination");
  if (o.csr != MISTIC_PAIRS_NONE && o.csr != MISTIC_PAIRS_HOST && o.csr != MISTIC_PAIRS_DEVICE)
    throw Error(MISTIC_ERR_INVALID_ARG, "unknown csr destination");
  if (o.input_on_device && n > 0) {
    cudaPointerAttributes pa;
    MCK(cudaPointerGetAttributes(&pa, pts));
    if (pa.type != cudaMemoryTypeDevice && pa.type != cudaMemoryTypeManaged)
      throw Error(MISTIC_ERR_INVALID_ARG, "input_on_device set but pts is not device memory");
  }
  const uint32_t launches0 = h->launches;
  r->n = n;
  r->d = d;
  r->mode_used = o.mode;
  if (n <= 1) {
    r->pairs_ordered_incl_self = n;
    if (o.csr != MISTIC_PAIRS_NONE) {  // a lone point is its own neighbour
      uint64_t off[2] = {0, n};
      uint32_t nb[1] = {0};
      if (o.csr == MISTIC_PAIRS_HOST) {
        r->csr_offsets = (uint64_t*)malloc(sizeof off);
        r->csr_nbrs = (uint32_t*)malloc(sizeof nb);
        if (!r->csr_offsets || !r->csr_nbrs) throw Error(MISTIC_ERR_OUT_OF_MEMORY, "host csr");
        memcpy(r->csr_offsets, off, (n + 1) * sizeof(uint64_t));
        memcpy(r->csr_nbrs, nb, sizeof nb);
      } else {
        MCK(cudaMalloc((void**)&r->csr_offsets, sizeof off));
        MCK(cudaMalloc((void**)&r->csr_nbrs, sizeof nb));
        MCK(cudaMemcpy(r->csr_offsets, off, (n + 1) * sizeof(uint64_t), cudaMemcpyHostToDevice));
        MCK(cudaMemcpy(r->csr_nbrs, nb, sizeof nb, cudaMemcpyHostToDevice));
        r->csr_on_device = 1;
      }
    }
    r->ms_wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    return;
  }
  const size_t esz = dt == MISTIC_F64 ? 8 : 4;
  PhaseClock clk{h, o.timing != 0};
  clk.mark();  // 0

  // ---- input on the device
  const void* x = pts;
  if (!o.input_on_device) {
    void* dx = h->arena.get("raw", n * d * esz);
    h2d(h, dx, pts, n * d * esz);
    x = dx;
  }
  clk.mark();  // 1

  // ---- column statistics (+ finiteness) and, for PCA points, a sample covariance
  const uint32_t cs_parts = (uint32_t)std::min<uint64_t>(std::max<uint64_t>(1, n / 2048), 1024);
  double* cs_part = abuf<double>(h, "cs_part", (size_t)cs_parts * 3 * d);
  double* cs_out = abuf<double>(h, "cs_out", 3 * (size_t)d);
  unsigned* flag = abuf<unsigned>(h, "flag", 4);
  MCK(cudaMemsetAsync(flag, 0, 4 * sizeof(unsigned), h->stream));
  idx::colstats(h, x, dt, n, d, cs_part, cs_parts, cs_out, flag);
  const bool scored = o.rp_mode == MISTIC_RP_SCORED && k > 0 && d >= 2 && d <= 1024;
  const bool pca = (o.rp_mode == MISTIC_RP_PCA || scored) && k > 0 && d >= 2 && d <= 1024;
  const uint32_t S = (uint32_t)std::min<uint64_t>(n, d <= 64 ? 8192 : 4096);
  double* cov = nullptr;
  double* sbuf = nullptr;
  if (pca) {
    sbuf = abuf<double>(h, "sample", (size_t)S * d);
    cov = abuf<double>(h, "cov", (size_t)d * d);
    double* cpart = abuf<double>(h, "cov_part", (size_t)((S + 127) / 128) * d * d);
    idx::sample_cov(h, x, dt, n, d, S, sbuf, cs_out /* full-data column means */, cpart, cov);
  }
  std::vector<double> stats(3 * (size_t)d);
  unsigned nonfinite = 0;
  d2h(h, stats.data(), cs_out, stats.size() * sizeof(double));
  d2h(h, &nonfinite, flag, sizeof(unsigned));
  if (nonfinite && o.check_finite) throw Error(MISTIC_ERR_NOT_FINITE, "input holds NaN or infinite coordinates");
  std::vector<double> mean(stats.begin(), stats.begin() + d), mn(stats.begin() + d, stats.begin() + 2 * d),
      mx(stats.begin() + 2 * d, stats.end());
  std::vector<double> covh;
  if (pca) {
    covh.resize((size_t)d * d);
    d2h(h, covh.data(), cov, covh.size() * sizeof(double));
  }
  std::vector<double> rps;
  if (scored) {
    std::vector<double> sh((size_t)S * d);
    d2h(h, sh.data(), sbuf, sh.size() * sizeof(double));
    select_reference_points_scored(o, d, k, eps, mean, mn, mx, covh, sh, S, rps);
  } else {
    select_reference_points(o, d, k, mean, mn, mx, covh, rps);
  }
  clk.mark();  // 2

  // ---- FP64 reference-point distances, key layout, packed keys
  const uint32_t kk = k;
  double* Dk = nullptr;
  PackParams pp{};
  EnumParams ep{};
  int total_bits = 0, k_used = 0;
  const double eps2 = eps * eps;
  if (kk > 0) {
    double* drp = abuf<double>(h, "rps", (size_t)kk * d);
    h2d(h, drp, rps.data(), rps.size() * sizeof(double));
    Dk = abuf<double>(h, "rpdist", n * kk);
    const uint32_t nparts = (uint32_t)((n + 255) / 256);
    double* part = abuf<double>(h, "rp_part", (size_t)nparts * 2 * kk);
    double* mm = abuf<double>(h, "rp_mm", 2 * (size_t)kk);
    idx::rp_dist(h, x, dt, n, d, drp, (int)kk, Dk, part, nparts, mm);
    std::vector<double> mmh(2 * (size_t)kk);
    d2h(h, mmh.data(), mm, mmh.size() * sizeof(double));
    // Field widths.  δ covers the FP64 error of the distances (relative
    // (d/2+2)u each), of the difference D - Dmin, and of the quotient.
    int fields = 0;
    int bits_acc = 0;
    int fb[MAX_K];
    for (uint32_t j = 0; j < kk; ++j) {
      const double dmin = mmh[j], dmax = mmh[kk + j];
      // distances that overflow FP64 (coordinates near 1e300) or a reference
      // point that is not finite: the field cannot bin, so it is dropped and
      // all points share it (the ±1 guarantee needs finite fields)
      if (!std::isfinite(dmin) || !std::isfinite(dmax) || !(dmax >= dmin)) continue;
      const double u64 = ldexp(1.0, -53);
      const double ratio = eps > 0 ? dmax / eps : 0.0;
      const double delta = std::max(ldexp(1.0, -20), 8.0 * (d + 4) * u64 * (1.0 + ratio));
      double w = eps * (1.0 + delta);
      const double span = dmax - dmin;
      if (!(w > 0) || span / w > ldexp(1.0, 30)) w = std::max(w, span / ldexp(1.0, 30));
      if (!(w > 0)) w = 1.0;  // all distances equal: a single field value
      const double mk = std::min(floor(span / w), ldexp(1.0, 30));
      if (mk < 1.0) continue;  // uninformative field: every point in the same slot
      const uint32_t maxkey = (uint32_t)mk;
      const int b = bit_length(maxkey);
      if (bits_acc + b > KEY_BITS_MAX) break;
      pp.col[fields] = (int)j;
      pp.dmin[fields] = dmin;
      pp.w[fields] = w;
      pp.maxkey[fields] = maxkey;
      ep.maxkey[fields] = maxkey;
      fb[fields] = b;
      bits_acc += b;
      ++fields;
    }
    k_used = fields;
    total_bits = bits_acc;
    // field 0 is the most significant
    int sh = total_bits;
    for (int f = 0; f < fields; ++f) {
      sh -= fb[f];
      pp.shift[f] = sh;
      ep.shift[f] = sh;
    }
    pp.k = fields;
    pp.kstride = (int)kk;
    ep.k = fields;
  }
  r->k_used = (uint32_t)k_used;
  uint64_t* keys[2] = {abuf<uint64_t>(h, "keys0", n), abuf<uint64_t>(h, "keys1", n)};
  uint32_t* vals[2] = {abuf<uint32_t>(h, "vals0", n), abuf<uint32_t>(h, "vals1", n)};
  if (k_used > 0) {
    idx::pack_keys(h, Dk, n, pp, keys[0]);
  } else {
    MCK(cudaMemsetAsync(keys[0], 0, n * sizeof(uint64_t), h->stream));
  }
  clk.mark();  // 3

  // ---- sort points by key
  int cur = 0;
  if (total_bits > 0) {
    cur = radix_sort_u64(h, keys, vals, true, true, n, total_bits);
  } else {
    idx::iota(h, vals[0], n);
  }
  const uint64_t* skeys = keys[cur];
  const uint32_t* perm = vals[cur];
  clk.mark();  // 4

  // ---- bins
  uint32_t* flags = abuf<uint32_t>(h, "binflags", n);
  uint32_t* nb_dev = abuf<uint32_t>(h, "nbins", 1);
  uint32_t* bstart = abuf<uint32_t>(h, "bstart", n + 1);
  uint64_t* bkey = abuf<uint64_t>(h, "bkey", n);
  idx::bins(h, skeys, n, flags, nb_dev, bstart, bkey);
  uint32_t m = 0;
  d2h(h, &m, nb_dev, sizeof(uint32_t));
  r->n_bins = m;

  // ---- mode and sorted-order gather
  bool fp64 = (o.mode == MISTIC_MODE_FP64);
  const uint32_t dpad32 = (d + 3) & ~3u, dpad64 = (d + 1) & ~1u;
  std::vector<double> center(d, 0.0);
  if (!fp64)
    for (uint32_t i = 0; i < d; ++i) center[i] = 0.5 * (mn[i] + mx[i]);
  double* dcenter = abuf<double>(h, "center", d);
  h2d(h, dcenter, center.data(), d * sizeof(double));
  uint32_t* ids = abuf<uint32_t>(h, "ids", n);
  float* xf = fp64 ? nullptr : abuf<float>(h, "xf", n * dpad32);
  double* xd = fp64 ? abuf<double>(h, "xd", n * dpad64) : nullptr;
  const uint32_t gparts = (uint32_t)((n + 255) / 256);
  double* npart = abuf<double>(h, "norm_part", gparts);
  double* rmax = abuf<double>(h, "rmax", 1);
  idx::gather(h, x, dt, n, d, perm, dcenter, fp64 ? 0 : dpad32, xf, fp64 ? dpad64 : 0, xd, ids, npart, rmax);
  double R2 = 0;
  d2h(h, &R2, rmax, sizeof(double));
  const double R = sqrt(R2) * (1.0 + 1e-12);
  float t_lo = 0, t_hi = 0;
  if (!fp64) {
    // FP32 range guard: fall back to the FP64 join when FP32 cannot hold the
    // coordinates or ε² comfortably.
    if (R > 1e15 || (eps2 > 0 && eps2 < 1e-28) || eps2 == 0.0 ||
        !filter_thresholds(d, eps2, R, &t_lo, &t_hi)) {
      fp64 = true;
      xd = abuf<double>(h, "xd", n * dpad64);
      idx::gather(h, x, dt, n, d, perm, dcenter, 0, nullptr, dpad64, xd, ids, npart, rmax);
    }
  }
  // tensor cores for large home bins when the FP32 view is usable and the
  // augmented K fits one operand tile
  // AUTO takes the tensor cores from d = 8 up (measured faster than the FP32
  // filter on the 5M x 18 join); below that the augmented K is mostly padding
  const bool tf32_mode = o.mode == MISTIC_MODE_TF32;
  const bool use_tc = !fp64 && join::tc_supported(d) && eps2 > 1e-20 &&
                      (o.mode == MISTIC_MODE_BF16 || tf32_mode || (o.mode == MISTIC_MODE_AUTO && d >= 8));
  // long rows (augmented K above one 128-wide operand tile), and every row in
  // tf32 mode, use the K-chunked kernel over rows prepared once; its operand
  // precision is picked from the bound (see tc_precision)
  // (the fused batch join drains medium rows with the short-row kernel only)
  const bool wide = use_tc && (tf32_mode || join::tc_kp(d) > 128 || (!ex && tcw_for_medium_rows(d, eps2, R)));
  const int prec = wide ? tc_precision(o.mode, d, eps2, R) : 0;
  r->mode_used = fp64 ? MISTIC_MODE_FP64
                      : (use_tc ? (tf32_mode ? MISTIC_MODE_TF32 : MISTIC_MODE_BF16) : MISTIC_MODE_FP32);
  clk.mark();  // 5

  // ---- neighbour enumeration -> work units
  const int CH = join::chunk_for(fp64, fp64 ? dpad64 : dpad32);
  ep.chunk = (uint32_t)CH;
  ep.seg_cap = 4096;
  // tensor-core units of large joins take longer segments: each unit reloads
  // and converts its home rows and drains the tile pipeline once, which cost
  // 4 ms of the 5M x 18 join at 4096 points against 16384; small joins keep
  // short segments so that the persistent grid has units enough to balance,
  // and the pair ring keeps them so that a unit's pairs fit it
  ep.seg_cap_tc = (n >= (1u << 20) && o.ring_capacity == 0) ? 16384u : 4096u;
  if (const char* e = getenv("MISTIC_SEG_CAP_TC")) ep.seg_cap_tc = (uint32_t)std::max(128l, strtol(e, nullptr, 10));
  ep.sample = o.home_sample;
  ep.tc_min = use_tc ? tc_min_bin(d, wide) : 0u;
  ep.tc_chunk = use_tc ? (wide ? 256u : join::tc_rows(d)) : 128;
  // prefix table of the enumeration: the first p <= 5 key fields (3^p
  // lookups a bin) while the table stays within 16 entries a bin and 2^24
  {
    const unsigned long long lim = std::min<unsigned long long>(1ull << 24, 16ull * m + 4096);
    unsigned long long entries = 1;
    int p = 0;
    while (p < std::min(ep.k, 5) && entries * (ep.maxkey[p] + 1ull) <= lim) entries *= ep.maxkey[p] + 1ull, ++p;
    ep.p = p;
    ep.ptab = nullptr;
    if (p > 0) {
      uint32_t st = 1;
      for (int j = p - 1; j >= 0; --j) {
        ep.stride[j] = st;
        st *= ep.maxkey[j] + 1u;
      }
      uint32_t* ptab = abuf<uint32_t>(h, "ptab", (size_t)entries + 1);
      idx::prefix_table(h, bkey, m, ep, ptab, (uint32_t)entries);
      ep.ptab = ptab;
    }
  }
  uint32_t tots[3] = {0, 0, 0};
  unsigned long long totc = 0;
  uint32_t* nbr = nullptr;
  Unit* units = nullptr;
  Unit* units_tc = nullptr;
  // count -> 64-bit totals check -> scans -> fill, into the arena's work lists
  auto enumerate_units = [&](const EnumParams& e) {
    uint32_t* nbr_cnt = abuf<uint32_t>(h, "nbr_cnt", m + 1);
    uint32_t* unit_cnt = abuf<uint32_t>(h, "unit_cnt", m + 1);
    uint32_t* unit_cnt_tc = abuf<uint32_t>(h, "unit_cnt_tc", m + 1);
    unsigned long long* cand = abuf<unsigned long long>(h, "cand", m + 1);
    idx::enumerate(h, bkey, bstart, m, e, nbr_cnt, unit_cnt, unit_cnt_tc, cand, nullptr, nullptr, nullptr, nullptr,
                   nullptr, nullptr, false);
    uint32_t* tot32 = abuf<uint32_t>(h, "tot32", 3);
    unsigned long long* tot64 = abuf<unsigned long long>(h, "tot64", 4);
    // 64-bit totals first: the work lists index neighbours and units with
    // 32-bit offsets, which a total of 2^32 or more would wrap
    idx::count_totals(h, nbr_cnt, unit_cnt, unit_cnt_tc, m, tot64 + 1);
    exclusive_scan<uint32_t>(h, nbr_cnt, nbr_cnt, m, tot32);
    exclusive_scan<uint32_t>(h, unit_cnt, unit_cnt, m, tot32 + 1);
    exclusive_scan<uint32_t>(h, unit_cnt_tc, unit_cnt_tc, m, tot32 + 2);
    exclusive_scan<unsigned long long>(h, cand, cand, m, tot64);
    unsigned long long tot_all[4] = {0, 0, 0, 0};
    d2h(h, tots, tot32, sizeof tots);
    d2h(h, tot_all, tot64, sizeof tot_all);
    totc = tot_all[0];
    // MISTIC_TEST_WORKLIST_LIMIT=k lowers the limit (tests of this check)
    unsigned long long lim = 0xffffffffull - 1;
    if (const char* ev = getenv("MISTIC_TEST_WORKLIST_LIMIT")) lim = std::min(lim, strtoull(ev, nullptr, 10));
    for (int i = 0; i < 3; ++i)
      if (tot_all[1 + i] > lim || tot_all[1 + i] != (unsigned long long)tots[i])
        throw Error(MISTIC_ERR_TOO_LARGE,
                    "neighbour-bin or work-unit list beyond the 32-bit offsets of the join work lists "
                    "(raise eps resolution: more reference points, or split the input)");
    nbr = abuf<uint32_t>(h, "nbr", (size_t)tots[0] + 1);
    units = abuf<Unit>(h, "units", (size_t)tots[1] + 1);
    units_tc = abuf<Unit>(h, "units_tc", (size_t)tots[2] + 1);
    idx::enumerate(h, bkey, bstart, m, e, nullptr, nullptr, nullptr, nullptr, nbr_cnt, unit_cnt, unit_cnt_tc, nbr,
                   units, units_tc, true);
  };

  // ---- join parameters
  JoinParams jp{};
  jp.bstart = bstart;
  jp.ids = ids;
  jp.xs = fp64 ? (const void*)xd : (const void*)xf;
  jp.dpad = fp64 ? dpad64 : dpad32;
  jp.raw = x;
  jp.raw_f32 = dt == MISTIC_F32;
  jp.d = d;
  jp.t_lo = t_lo;
  jp.t_hi = t_hi;
  jp.eps2 = eps2;
  jp.amb = 4.0 * (nextafter(eps2, INFINITY) - eps2);
  JoinCounters* ctr = abuf<JoinCounters>(h, "ctr", 2);  // [0] CUDA-core join, [1] tensor-core cursor
  jp.ctr = ctr;
  if (!fp64) {  // band pairs are pre-decided with the FP32 filter on the sorted FP32 rows
    uint32_t* inv = abuf<uint32_t>(h, "inv", n);
    k_inverse_perm<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(ids, n, inv);
    launched(h, "inverse_perm");
    jp.inv = inv;
    jp.xf32 = xf;
    jp.dpad32 = dpad32;
  }
  TcParams tp{};
  int prepared = -1;  // operand precision the K-chunked kernel's rows are prepared at
  // tensor-core parameters at operand precision pr (rows prepared on demand)
  auto set_tc = [&](int pr) {
    if (!use_tc) return;
    const double u = ldexp(1.0, -24) * (1.0 + ldexp(1.0, -20));
    const double gd = d * u / (1.0 - d * u);
    const double g64 = (d + 2) * ldexp(1.0, -53) * 1.01;
    tp.ctr = ctr + 1;
    tp.b.eps2_lo = (float)(eps2 / (1.0 + g64));
    if ((double)tp.b.eps2_lo > eps2 / (1.0 + g64)) tp.b.eps2_lo = nextafterf(tp.b.eps2_lo, 0.f);
    tp.b.eps2_hi = (float)(eps2 / (1.0 - g64));
    if ((double)tp.b.eps2_hi < eps2 / (1.0 - g64)) tp.b.eps2_hi = nextafterf(tp.b.eps2_hi, INFINITY);
    tp.b.kappa = (float)tc_kappa(d, wide, pr);
    tp.b.ginf = (float)(1.0 / (1.0 - gd) * (1.0 + 1e-6));
    tp.b.uR2 = (float)(2.0 * u * R * 1.0001);
    tp.b.u1 = (float)(u * (1.0 + u) * 1.0001);
    tp.b.Dp = (float)(1.1 * sqrt(eps2));
    tp.b.cap = (float)(0.1 * eps2);
    tp.b.margin = (float)(1e-6 * eps2);
    // MISTIC_TEST_TC_STALL=1 is the failure-detection test: the MMA warp
    // signals nothing, every bounded wait runs out after a short limit, the
    // kernel frees its tensor memory and the call returns MISTIC_ERR_TIMEOUT
    const char* st = getenv("MISTIC_TEST_TC_STALL");
    tp.stall_test = (st && *st == '1') ? 1 : 0;
    tp.wait_limit = tp.stall_test ? 2000000ll : 2000000000ll;  // 2 ms in the test, else 2 s
    tp.prof = getenv("MISTIC_DEBUG") ? 1 : 0;
    tp.prec = pr;
    if (wide && prepared != pr) {
      tp.kd = join::tcw_kd(d, pr);
      // operand rows: bf16 (hi, and lo for the split) or tf32 in FP32 words
      void* xh = h->arena.get("xh", n * (size_t)tp.kd * (pr == 2 ? 4 : 2));
      void* xl = pr == 0 ? h->arena.get("xl", n * (size_t)tp.kd * 2) : nullptr;
      float* xn = abuf<float>(h, "xn", n);
      join::tcw_prepare(h, pr, xf, dpad32, d, n, xh, xl, xn);
      tp.xh = xh;
      tp.xl = xl;
      tp.xn = xn;
      tp.n_rows = n;
      prepared = pr;
    }
  };
  auto point_lists = [&]() {
    jp.units = units;
    jp.n_units = tots[1];
    jp.nbr = nbr;
    tp.units = units_tc;
    tp.n_units = tots[2];
  };
  // one pass of the join kernels: CUDA cores, tensor cores, FP64 band decisions
  auto launch_join = [&](bool timed) {
    MCK(cudaMemsetAsync(ctr, 0, 2 * sizeof(JoinCounters), h->stream));
    if (timed) MCK(cudaEventRecord(h->jev[0], h->stream));
    join::run(h, fp64, CH, jp);
    if (timed) MCK(cudaEventRecord(h->jev[1], h->stream));
    if (use_tc) {
      if (wide)
        join::run_tcw(h, jp, tp);
      else
        join::run_tc(h, jp, tp);
    }
    if (timed) MCK(cudaEventRecord(h->jev[2], h->stream));
    join::run_band(h, jp);
    if (timed) MCK(cudaEventRecord(h->jev[3], h->stream));
  };
  // band list: pairs the FP32 / tensor-core joins leave to the FP64 check
  auto size_band = [&](unsigned long long cands) {
    if (fp64) return;
    // measured band fractions are ~2e-5 - 5e-5 of the candidate pairs; start
    // above that so the first call rarely has to run the join again
    unsigned long long bcap = std::max<unsigned long long>(1ull << 20, 2ull * n);
    bcap = std::max<unsigned long long>(bcap, std::min<unsigned long long>(cands / 8192, 1ull << 30));
    auto it = h->arena.bufs.find("band");
    if (it != h->arena.bufs.end()) bcap = std::max<unsigned long long>(bcap, it->second.bytes / 8);
    // MISTIC_BAND_CAP=k starts from a k-entry list (tests of the overflow path)
    if (const char* e = getenv("MISTIC_BAND_CAP")) bcap = std::max<unsigned long long>(1, strtoull(e, nullptr, 10));
    jp.band_list = abuf<unsigned long long>(h, "band", bcap);
    jp.band_cap = bcap;
  };

  // ---- autotuner: tensor-core bin threshold (and, for the K-chunked kernel,
  // the operand precision) timed on a sample of the work, once per shape
  int prec_used = prec;
  if (use_tc && !tf32_mode) {
    Tuned tu;
    if (tune_lookup(h, o, d, dt, wide, prec, bstart, m, eps2, R, &tu, [&](const TuneCandidate& c, uint32_t S,
                                                                           double* ms_out, unsigned long long* cands,
                                                                           unsigned long long* nunits) {
          EnumParams e2 = ep;
          e2.tc_min = c.tc_min;
          e2.sample = std::max<uint32_t>(S, o.home_sample);
          enumerate_units(e2);
          set_tc(c.prec);
          point_lists();
          jp.pairs = nullptr;
          jp.cap = 0;
          size_band(totc);
          launch_join(true);
          JoinCounters hc2{};
          d2h(h, &hc2, ctr, sizeof hc2);
          if (hc2.error) throw Error(MISTIC_ERR_TIMEOUT, "a tensor-core tile wait timed out");
          float t = 0;
          MCK(cudaEventElapsedTime(&t, h->jev[0], h->jev[3]));
          *ms_out = t;
          *cands = totc;
          // the sample must give each join enough units to balance the
          // persistent grid (tensor-core units are long and few): the
          // smaller of the two counts decides
          const unsigned long long us = tots[1], ut = tots[2];
          *nunits = (us && ut) ? std::min(us, ut) : us + ut;
        })) {
      ep.tc_min = tu.tc_min;
      prec_used = tu.prec;
      r->tuned = 1;
    }
  }
  r->tc_min_bin = ep.tc_min;
  enumerate_units(ep);
  r->n_bin_pairs = tots[0];
  r->n_units = tots[1];
  r->n_units_tc = tots[2];
  r->candidates = totc;
  clk.mark();  // 6

  // ---- join
  set_tc(prec_used);
  point_lists();
  if (ex && !fp64 && !wide && ex->alloc) {
    // ---- fused batch: hand the work lists over instead of joining
    const size_t b_xf = n * (size_t)dpad32 * sizeof(float), b_ids = n * sizeof(uint32_t),
                 b_bs = ((size_t)m + 1) * sizeof(uint32_t), b_nbr = ((size_t)tots[0] + 1) * sizeof(uint32_t),
                 b_u = ((size_t)tots[1] + 1) * sizeof(Unit), b_ut = ((size_t)tots[2] + 1) * sizeof(Unit);
    // host input: its device copy lives in this handle's arena, so it moves too
    const size_t b_raw = o.input_on_device ? 0 : n * d * esz;
    auto al = [](size_t b) { return (b + 255) & ~(size_t)255; };
    unsigned char* base = (unsigned char*)ex->alloc(al(b_xf) + al(b_ids) + al(b_bs) + al(b_nbr) + al(b_u) +
                                                    al(b_ut) + al(b_raw));
    if (base) {
      unsigned char* p = base;
      float* e_xf = (float*)p;
      p += al(b_xf);
      uint32_t* e_ids = (uint32_t*)p;
      p += al(b_ids);
      uint32_t* e_bs = (uint32_t*)p;
      p += al(b_bs);
      uint32_t* e_nbr = (uint32_t*)p;
      p += al(b_nbr);
      Unit* e_u = (Unit*)p;
      p += al(b_u);
      Unit* e_ut = (Unit*)p;
      p += al(b_ut);
      const void* e_raw = x;
      if (b_raw) {
        MCK(cudaMemcpyAsync(p, x, b_raw, cudaMemcpyDeviceToDevice, h->stream));
        e_raw = p;
      }
      MCK(cudaMemcpyAsync(e_xf, xf, b_xf, cudaMemcpyDeviceToDevice, h->stream));
      k_add_u32<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(ids, e_ids, n, ex->row0);
      launched(h, "add_u32");
      MCK(cudaMemcpyAsync(e_bs, bstart, b_bs, cudaMemcpyDeviceToDevice, h->stream));
      MCK(cudaMemcpyAsync(e_nbr, nbr, (size_t)tots[0] * sizeof(uint32_t), cudaMemcpyDeviceToDevice, h->stream));
      if (tots[1]) MCK(cudaMemcpyAsync(e_u, units, (size_t)tots[1] * sizeof(Unit), cudaMemcpyDeviceToDevice, h->stream));
      if (tots[2])
        MCK(cudaMemcpyAsync(e_ut, units_tc, (size_t)tots[2] * sizeof(Unit), cudaMemcpyDeviceToDevice, h->stream));
      InstDesc& D = ex->desc;
      D.bstart = e_bs;
      D.nbr = e_nbr;
      D.ids = e_ids;
      D.xs = e_xf;
      D.raw = e_raw;
      D.d = d;
      D.raw_f32 = dt == MISTIC_F32;
      D.row0 = ex->row0;
      D.t_lo = t_lo;
      D.t_hi = t_hi;
      D.eps2 = eps2;
      D.amb = jp.amb;
      D.tcb = tp.b;
      ex->dpad32 = dpad32;
      ex->units = e_u;
      ex->n_units = tots[1];
      ex->units_tc = e_ut;
      ex->n_units_tc = tots[2];
      ex->CH = CH;
      ex->exported = true;
      r->tc_operands = (use_tc && tots[2] > 0) ? 1 : 0;
      r->tc_kernel = (use_tc && tots[2] > 0) ? 1 : 0;
      MCK(cudaStreamSynchronize(h->stream));  // the arena is reused by this handle's next call
      r->ms_wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
      r->kernel_launches = h->launches - launches0;
      return;
    }
  }
  if (o.ring_capacity > 0) {
    // ---- streamed pair ring: passes of the join over a fixed ring
    if (o.csr != MISTIC_PAIRS_NONE || (o.pairs != MISTIC_PAIRS_HOST && !o.pair_sink))
      throw Error(MISTIC_ERR_INVALID_ARG, "the pair ring streams to host memory or a pair_sink (no CSR table)");
    const unsigned long long C = o.ring_capacity;
    const unsigned long long NT = (unsigned long long)tots[1] + tots[2];  // unit tags
    unsigned long long* ring = abuf<unsigned long long>(h, "ring", C);
    uint32_t* rtags = abuf<uint32_t>(h, "ring_tags", C);
    unsigned long long* rout = abuf<unsigned long long>(h, "ring_out", C);
    uint32_t* rdef = abuf<uint32_t>(h, "ring_deferred", NT + 1);
    uint32_t* rdef_out = abuf<uint32_t>(h, "ring_def_out", NT + 1);
    uint32_t* rdin_s = abuf<uint32_t>(h, "ring_def_in_s", (size_t)tots[1] + 1);
    uint32_t* rdin_t = abuf<uint32_t>(h, "ring_def_in_t", (size_t)tots[2] + 1);
    unsigned long long* rcount = abuf<unsigned long long>(h, "ring_count", 1);
    MCK(cudaMemsetAsync(rdef, 0, (NT + 1) * sizeof(uint32_t), h->stream));
    size_band(totc);
    uint32_t* btags = abuf<uint32_t>(h, "band_tags", jp.band_cap);
    unsigned long long* stage = (unsigned long long*)pinned_cache().acquire(C * 8);
    if (!stage) throw Error(MISTIC_ERR_OUT_OF_MEMORY, "pinned ring staging");
    std::vector<unsigned long long> all;  // drained pairs (i << 32 | j) when they go to the result
    unsigned long long total = 0, redone = 0, bandd = 0, amb = 0;
    uint32_t passes = 0;
    unsigned long long main_s = 0, main_t = 0;
    std::vector<uint32_t> din_s, din_t;
    // after a pass that finished no unit: grids halved down to one block,
    // then one unit per kernel (a block of many warps can still hold several
    // units whose pairs together overfill the ring)
    uint32_t gcap = 0;            // 0: full persistent grids
    unsigned long long ccap = 0;  // 0: no cap on claims
    jp.ring = 1;
    jp.pairs = ring;
    jp.cap = C;
    jp.pair_tags = rtags;
    jp.band_tags = btags;
    jp.deferred = rdef;
    jp.def_out = rdef_out;
    jp.tag_base_tc = tots[1];
    auto drain = [&](unsigned long long used) {
      used = std::min(used, C);
      if (!used) return;
      MCK(cudaMemsetAsync(rcount, 0, sizeof(unsigned long long), h->stream));
      k_ring_drain<<<(unsigned)((used + 255) / 256), 256, 0, h->stream>>>(ring, rtags, rdef, used, rout, rcount);
      launched(h, "ring_drain");
      unsigned long long cnt = 0;
      d2h(h, &cnt, rcount, sizeof cnt);
      if (!cnt) return;
      MCK(cudaMemcpyAsync(stage, rout, cnt * 8, cudaMemcpyDeviceToHost, h->stream));
      MCK(cudaStreamSynchronize(h->stream));
      total += cnt;
      if (o.pair_sink) {
        for (unsigned long long i = 0; i < cnt; ++i) stage[i] = (stage[i] >> 32) | (stage[i] << 32);  // (i, j)
        o.pair_sink((const uint32_t*)stage, cnt, o.sink_user);
      } else {
        all.insert(all.end(), stage, stage + cnt);
      }
    };
    mistic_status rs = MISTIC_OK;
    try {
      for (;;) {
        const bool left_s = main_s < tots[1] || !din_s.empty();
        const bool left_t = use_tc && (main_t < tots[2] || !din_t.empty());
        if (!left_s && !left_t) break;
        if (!din_s.empty())
          MCK(cudaMemcpyAsync(rdin_s, din_s.data(), din_s.size() * 4, cudaMemcpyHostToDevice, h->stream));
        if (!din_t.empty())
          MCK(cudaMemcpyAsync(rdin_t, din_t.data(), din_t.size() * 4, cudaMemcpyHostToDevice, h->stream));
        MCK(cudaMemsetAsync(ctr, 0, 2 * sizeof(JoinCounters), h->stream));
        jp.def_in = rdin_s;
        jp.n_def_in = (uint32_t)din_s.size();
        jp.main_start = main_s;
        jp.grid_cap = gcap;
        jp.claim_cap = ccap;
        tp.def_in = rdin_t;
        tp.n_def_in = (uint32_t)din_t.size();
        tp.main_start = main_t;
        tp.grid_cap = gcap;
        tp.claim_cap = ccap;
        if (left_s) join::run(h, fp64, CH, jp);
        if (left_t) {
          if (wide)
            join::run_tcw(h, jp, tp);
          else
            join::run_tc(h, jp, tp);
        }
        JoinCounters c0{}, c1{};
        d2h(h, &c0, ctr, sizeof c0);
        d2h(h, &c1, ctr + 1, sizeof c1);
        if (c0.error || c1.error) throw Error(MISTIC_ERR_TIMEOUT, "a tensor-core tile wait timed out");
        std::vector<uint32_t> dout(c0.def_n);
        if (c0.def_n) d2h(h, dout.data(), rdef_out, c0.def_n * 4);
        // the pairs of units that finished, then the band decisions of their
        // band entries in slices the ring can hold
        drain(c0.pairs);
        const unsigned long long nb = std::min(c0.band_n, jp.band_cap);
        for (unsigned long long b0 = 0; b0 < nb; b0 += C) {
          MCK(cudaMemsetAsync(&ctr[0].pairs, 0, sizeof(unsigned long long), h->stream));
          jp.band0 = b0;
          jp.band1 = std::min(nb, b0 + C);
          join::run_band(h, jp);
          unsigned long long used = 0;
          d2h(h, &used, &ctr[0].pairs, sizeof used);
          drain(used);
        }
        {
          JoinCounters cb{};
          d2h(h, &cb, ctr, sizeof cb);
          bandd += cb.band;
          amb += cb.ambiguous;
        }
        // cursors: claims past the deferred list came from the main list;
        // deferred units that were never claimed are carried over
        const unsigned long long cs = ccap ? std::min(c0.next_unit, ccap) : c0.next_unit;
        const unsigned long long ct = ccap ? std::min(c1.next_unit, ccap) : c1.next_unit;
        const unsigned long long nds = din_s.size(), ndt = din_t.size();
        const unsigned long long got_s = left_s ? std::min(cs, nds) + std::min(cs > nds ? cs - nds : 0ull, tots[1] - main_s) : 0;
        const unsigned long long got_t = left_t ? std::min(ct, ndt) + std::min(ct > ndt ? ct - ndt : 0ull, tots[2] - main_t) : 0;
        std::vector<uint32_t> ns(din_s.begin() + std::min(cs, nds), din_s.end());
        std::vector<uint32_t> nt(din_t.begin() + std::min(ct, ndt), din_t.end());
        if (!left_s) ns = din_s;
        if (!left_t) nt = din_t;
        if (left_s) main_s += std::min(cs > nds ? cs - nds : 0ull, tots[1] - main_s);
        if (left_t) main_t += std::min(ct > ndt ? ct - ndt : 0ull, tots[2] - main_t);
        for (uint32_t tg : dout) {
          if (tg < tots[1])
            ns.push_back(tg);
          else
            nt.push_back(tg - tots[1]);
        }
        if (c0.def_n) {
          MCK(cudaMemcpyAsync(rdef_out, dout.data(), dout.size() * 4, cudaMemcpyHostToDevice, h->stream));
          k_clear_flags<<<(unsigned)((c0.def_n + 255) / 256), 256, 0, h->stream>>>(rdef, rdef_out, c0.def_n);
          launched(h, "clear_flags");
        }
        redone += c0.def_n;
        ++passes;
        din_s.swap(ns);
        din_t.swap(nt);
        if (got_s + got_t <= c0.def_n) {  // no unit finished: fewer units at a time
          if (ccap == 1) throw Error(MISTIC_ERR_PAIR_OVERFLOW, "a work unit has more pairs than the pair ring holds");
          if (gcap == 1) ccap = 1;
          gcap = gcap ? std::max(1u, gcap / 2) : (unsigned)std::max(1, h->sms / 2);
        }
      }
    } catch (const Error& e) {
      pinned_cache().release(stage);
      throw;
    }
    pinned_cache().release(stage);
    (void)rs;
    clk.mark();  // 7
    r->pairs_ij = total;
    r->pairs_ordered_incl_self = 2 * total + n;
    r->band_pairs = fp64 ? 0 : bandd;
    r->ulp_ambiguous = amb;
    r->ring_passes = passes;
    r->ring_units_redone = redone;
    r->tc_operands = (use_tc && tots[2] > 0) ? (wide ? 1 + prec_used : 1) : 0;
    r->tc_kernel = (use_tc && tots[2] > 0) ? (wide ? 2 : 1) : 0;
    if (!o.pair_sink) {
      if (o.sort_pairs) std::sort(all.begin(), all.end());
      uint32_t* hp = (uint32_t*)pinned_cache().acquire(std::max<size_t>(1, all.size() * 8));
      if (!hp) hp = (uint32_t*)malloc(std::max<size_t>(1, all.size() * 8));
      if (!hp) throw Error(MISTIC_ERR_OUT_OF_MEMORY, "host pair buffer");
      for (size_t i = 0; i < all.size(); ++i) {
        hp[2 * i] = (uint32_t)(all[i] >> 32);
        hp[2 * i + 1] = (uint32_t)all[i];
      }
      r->pairs = hp;
      r->pairs_len = all.size();
      r->pairs_on_device = 0;
      r->_owner = hp;
    }
    clk.mark();  // 8
    MCK(cudaStreamSynchronize(h->stream));
    r->ms_h2d = clk.ms(0, 1);
    r->ms_prep = clk.ms(1, 2);
    r->ms_keys = clk.ms(2, 3);
    r->ms_sort = clk.ms(3, 4);
    r->ms_bins = clk.ms(4, 5);
    r->ms_enum = clk.ms(5, 6);
    r->ms_join = clk.ms(6, 7);
    r->ms_d2h = clk.ms(7, 8);
    r->ms_total = clk.ms(0, 8);
    r->kernel_launches = h->launches - launches0;
    r->ms_wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
    return;
  }
  const bool want_pairs = o.pairs != MISTIC_PAIRS_NONE;
  const bool want_csr = o.csr != MISTIC_PAIRS_NONE;
  const bool need_pairs = want_pairs || want_csr;  // the CSR table is built from the pair list
  unsigned long long cap = 0;
  unsigned long long* pbuf = nullptr;
  const bool caller_buf = want_pairs && o.pairs == MISTIC_PAIRS_DEVICE && o.pair_buffer;
  // A host pair list that needs no device-side pass (no sort, no CSR table)
  // is written by the join kernels straight into pinned host memory where the
  // CPU-GPU link is coherent: the stores cross the link while the join runs,
  // in the result's (i, j) order, and no copy follows the join.
  bool host_direct = want_pairs && o.pairs == MISTIC_PAIRS_HOST && !o.sort_pairs && !want_csr && h->host_pairs;
  PinnedHold hold;
  hold.stream = h->stream;
  auto host_list = [&](unsigned long long c) -> unsigned long long* {
    hold.reset();
    hold.p = pinned_cache().acquire(std::max<size_t>(8, c * 8));
    void* dp = nullptr;
    if (hold.p && cudaHostGetDevicePointer(&dp, hold.p, 0) == cudaSuccess) return (unsigned long long*)dp;
    cudaGetLastError();
    hold.reset();
    return nullptr;
  };
  if (caller_buf) {
    if (!o.pair_capacity) throw Error(MISTIC_ERR_INVALID_ARG, "pair_buffer needs pair_capacity > 0");
    if ((uintptr_t)o.pair_buffer % 8) throw Error(MISTIC_ERR_INVALID_ARG, "pair_buffer must be 8-byte aligned");
    cap = o.pair_capacity;
    pbuf = (unsigned long long*)o.pair_buffer;
  } else if (need_pairs) {
    cap = o.pair_capacity ? o.pair_capacity : std::max<unsigned long long>(1ull << 20, 16ull * n);
    if (host_direct) {
      if (!o.pair_capacity) cap = std::max<unsigned long long>(cap, h->host_pair_cap);
      pbuf = host_list(cap);
      host_direct = pbuf != nullptr;  // no pinned block: the device list and a copy
    }
    if (!host_direct) {
      auto it = h->arena.bufs.find("pairs");
      if (!o.pair_capacity && it != h->arena.bufs.end()) cap = std::max<unsigned long long>(cap, it->second.bytes / 8);
      pbuf = abuf<unsigned long long>(h, "pairs", cap);
    }
  }
  jp.pairs = pbuf;
  jp.cap = cap;
  jp.pairs_ij = host_direct ? 1 : 0;
  size_band(totc);
  JoinCounters hc{};
  // MISTIC_TEST_JOIN_ATTEMPTS=k caps the passes (tests of the exit check below)
  int attempts = 3;
  if (const char* e = getenv("MISTIC_TEST_JOIN_ATTEMPTS")) attempts = std::max(1, atoi(e));
  bool complete = false;
  for (int attempt = 0; attempt < attempts; ++attempt) {
    launch_join(o.timing != 0);
    d2h(h, &hc, ctr, sizeof hc);
    if (hc.error) throw Error(MISTIC_ERR_TIMEOUT, "a tensor-core tile wait timed out");
    if (hc.band_n > jp.band_cap) {  // band list overflowed: nothing beyond it was decided, run again
      jp.band_cap = hc.band_n + hc.band_n / 4;
      jp.band_list = abuf<unsigned long long>(h, "band", jp.band_cap);
      continue;
    }
    if (!need_pairs || hc.pairs <= cap || o.pair_capacity) {
      complete = true;
      break;
    }
    cap = hc.pairs;
    if (host_direct) {
      pbuf = host_list(cap);
      host_direct = pbuf != nullptr;
    }
    if (!host_direct) pbuf = abuf<unsigned long long>(h, "pairs", cap);
    jp.pairs = pbuf;
    jp.cap = cap;
    jp.pairs_ij = host_direct ? 1 : 0;
  }
  // the last pass must have decided every band pair and, with a library-sized
  // pair buffer, stored every pair; otherwise the counts are not a result
  if (!complete)
    throw Error(MISTIC_ERR_INTERNAL, "the join's band list or pair buffer still overflowed after its last pass");
  clk.mark();  // 7
  r->pairs_ij = hc.pairs;
  r->pairs_ordered_incl_self = 2 * hc.pairs + n;
  r->band_pairs = fp64 ? 0 : hc.band;
  r->ulp_ambiguous = hc.ambiguous;
  r->tc_operands = (use_tc && tots[2] > 0) ? (wide ? 1 + prec_used : 1) : 0;
  r->tc_kernel = (use_tc && tots[2] > 0) ? (wide ? 2 : 1) : 0;
  if (use_tc) {
    JoinCounters tcc{};
    d2h(h, &tcc, ctr + 1, sizeof tcc);
    r->tc_tiles = tcc.tiles;
    r->tc_cells = tcc.cells;
    if (tp.prof && tp.xh) {
      const double tot_p = (double)tcc.prof[1], tot_m = (double)tcc.prof[4], tot_e = (double)tcc.prof[6];
      fprintf(stderr,
              "[mistic] join_tcw roles: producers group setup %.1f%% stage wait %.1f%% issue %.1f%% publish %.1f%% | "
              "MMA wait-full %.1f%% wait-acc %.1f%% | epilogue wait %.1f%% | %llu stages\n",
              tot_p ? 100.0 * tcc.prof[7] / tot_p : 0.0, tot_p ? 100.0 * tcc.prof[0] / tot_p : 0.0,
              tot_p ? 100.0 * tcc.prof[9] / tot_p : 0.0, tot_p ? 100.0 * tcc.prof[14] / tot_p : 0.0,
              tot_m ? 100.0 * tcc.prof[2] / tot_m : 0.0, tot_m ? 100.0 * tcc.prof[3] / tot_m : 0.0,
              tot_e ? 100.0 * tcc.prof[5] / tot_e : 0.0, (unsigned long long)tcc.prof[12]);
    } else if (tp.prof) {
      const double tot_p = (double)tcc.prof[1], tot_m = (double)tcc.prof[4], tot_e = (double)tcc.prof[6];
      fprintf(stderr,
              "[mistic] join_tc roles: producers wait-for-free-stage %.1f%% | MMA wait-full %.1f%% wait-free-acc "
              "%.1f%% | epilogue wait-acc %.1f%%\n",
              tot_p ? 100.0 * tcc.prof[0] / tot_p : 0.0, tot_m ? 100.0 * tcc.prof[2] / tot_m : 0.0,
              tot_m ? 100.0 * tcc.prof[3] / tot_m : 0.0, tot_e ? 100.0 * tcc.prof[5] / tot_e : 0.0);
      fprintf(stderr,
              "[mistic] join_tc detail: producers unit %.1f%% window %.1f%% convert %.1f%% (rows-wait %.1f%%) | epilogue tmem-ld "
              "%.1f%% slow %.1f%% stage %.1f%% | %llu tiles, %llu accumulator tiles\n",
              tot_p ? 100.0 * tcc.prof[7] / tot_p : 0.0, tot_p ? 100.0 * tcc.prof[8] / tot_p : 0.0,
              tot_p ? 100.0 * tcc.prof[9] / tot_p : 0.0, tot_p ? 100.0 * tcc.prof[14] / tot_p : 0.0,
              tot_e ? 100.0 * tcc.prof[10] / tot_e : 0.0,
              tot_e ? 100.0 * tcc.prof[11] / tot_e : 0.0, tot_e ? 100.0 * tcc.prof[13] / tot_e : 0.0,
              (unsigned long long)tcc.tiles, (unsigned long long)tcc.prof[12]);
      fprintf(stderr,
              "[mistic] join_tc producer steps (thread 0): advance %.1f%% | stage wait + barrier %.1f%% | pass 1 + "
              "norm + threshold %.1f%% | pass 2 %.1f%% | metadata + fence + arrive %.1f%%\n",
              tot_p ? 100.0 * tcc.prof[16] / tot_p : 0.0, tot_p ? 100.0 * tcc.prof[17] / tot_p : 0.0,
              tot_p ? 100.0 * tcc.prof[18] / tot_p : 0.0, tot_p ? 100.0 * tcc.prof[19] / tot_p : 0.0,
              tot_p ? 100.0 * tcc.prof[20] / tot_p : 0.0);
    }
  }

  // ---- CSR neighbour table (from the packed pair list, before it is sorted or converted)
  mistic_status tail = MISTIC_OK;
  if (want_csr) {
    const unsigned long long np = std::min<unsigned long long>(hc.pairs, cap);
    if (hc.pairs > cap) tail = MISTIC_ERR_PAIR_OVERFLOW;
    const unsigned long long E = 2 * np + n;
    if (E >= 0xffffffffull) throw Error(MISTIC_ERR_TOO_LARGE, "neighbour table beyond 2^32 entries");
    uint64_t* ek[2] = {abuf<uint64_t>(h, "csr_e0", E), abuf<uint64_t>(h, "csr_e1", E)};
    csr_edges(h, pbuf, np, n, (unsigned long long*)ek[0]);
    uint32_t* ev[2] = {nullptr, nullptr};
    const int c = radix_sort_u64(h, ek, ev, false, false, E, 32 + std::max(1, bit_length(n - 1)));
    uint64_t* offs = abuf<uint64_t>(h, "csr_off", n + 1);
    uint32_t* nbs = abuf<uint32_t>(h, "csr_nbr", E);
    csr_split(h, (const unsigned long long*)ek[c], E, nbs, (unsigned long long*)offs, n);
    if (o.csr == MISTIC_PAIRS_HOST) {
      r->csr_offsets = (uint64_t*)malloc((n + 1) * sizeof(uint64_t));
      r->csr_nbrs = (uint32_t*)malloc(std::max<size_t>(1, E * sizeof(uint32_t)));
      if (!r->csr_offsets || !r->csr_nbrs) throw Error(MISTIC_ERR_OUT_OF_MEMORY, "host csr table");
      MCK(cudaMemcpyAsync(r->csr_offsets, offs, (n + 1) * sizeof(uint64_t), cudaMemcpyDeviceToHost, h->stream));
      MCK(cudaMemcpyAsync(r->csr_nbrs, nbs, E * sizeof(uint32_t), cudaMemcpyDeviceToHost, h->stream));
      MCK(cudaStreamSynchronize(h->stream));
    } else {
      h->arena.bufs.erase("csr_off");  // the result owns them now
      h->arena.bufs.erase("csr_nbr");
      r->csr_offsets = offs;
      r->csr_nbrs = nbs;
      r->csr_on_device = 1;
    }
  }
  // ---- pair list
  if (want_pairs && host_direct) {
    const unsigned long long stored = std::min<unsigned long long>(hc.pairs, cap);
    if (hc.pairs > cap) tail = MISTIC_ERR_PAIR_OVERFLOW;
    h->host_pair_cap = std::max(h->host_pair_cap, cap);
    r->pairs = (uint32_t*)hold.p;  // the join's stores completed with its last kernel (synchronised above)
    r->pairs_len = stored;
    r->pairs_on_device = 0;
    r->_owner = hold.p;
    hold.p = nullptr;
  } else if (want_pairs) {
    const unsigned long long stored = std::min<unsigned long long>(hc.pairs, cap);
    if (hc.pairs > cap) tail = MISTIC_ERR_PAIR_OVERFLOW;
    if (o.sort_pairs && stored > 1) {
      uint64_t* pk[2] = {(uint64_t*)pbuf, abuf<uint64_t>(h, "pairs_tmp", stored)};
      uint32_t* pv[2] = {nullptr, nullptr};
      const int bits = bit_length(n - 1);
      int c = radix_sort_u64(h, pk, pv, false, false, stored, 32 + bits);
      if (c == 1) MCK(cudaMemcpyAsync(pbuf, pk[1], stored * 8, cudaMemcpyDeviceToDevice, h->stream));
    }
    pairs_to_ij(h, pbuf, stored);
    r->pairs_len = stored;
    if (o.pairs == MISTIC_PAIRS_HOST) {
      uint32_t* hp = (uint32_t*)pinned_cache().acquire(std::max<size_t>(1, stored * 8));
      if (!hp) hp = (uint32_t*)malloc(std::max<size_t>(1, stored * 8));
      if (!hp) throw Error(MISTIC_ERR_OUT_OF_MEMORY, "host pair buffer");
      MCK(cudaMemcpyAsync(hp, pbuf, stored * 8, cudaMemcpyDeviceToHost, h->stream));
      MCK(cudaStreamSynchronize(h->stream));
      r->pairs = hp;
      r->pairs_on_device = 0;
      r->_owner = (void*)hp;
    } else if (caller_buf) {
      r->pairs = o.pair_buffer;  // caller keeps ownership
      r->pairs_on_device = 1;
      r->_owner = nullptr;
    } else {
      // hand the device buffer to the result; the arena forgets it
      h->arena.bufs.erase("pairs");
      r->pairs = (uint32_t*)pbuf;
      r->pairs_on_device = 1;
      r->_owner = (void*)pbuf;
    }
  }
  clk.mark();  // 8
  MCK(cudaStreamSynchronize(h->stream));
  r->ms_h2d = clk.ms(0, 1);
  r->ms_prep = clk.ms(1, 2);
  r->ms_keys = clk.ms(2, 3);
  r->ms_sort = clk.ms(3, 4);
  r->ms_bins = clk.ms(4, 5);
  r->ms_enum = clk.ms(5, 6);
  r->ms_join = clk.ms(6, 7);
  r->ms_d2h = clk.ms(7, 8);
  r->ms_total = clk.ms(0, 8);
  if (o.timing) {
    float a = 0, b = 0;
    MCK(cudaEventElapsedTime(&a, h->jev[0], h->jev[1]));
    MCK(cudaEventElapsedTime(&b, h->jev[1], h->jev[2]));
    r->ms_join_simt = a;
    r->ms_join_tc = b;
  }
  r->kernel_launches = h->launches - launches0;
  r->ms_wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  if (tail != MISTIC_OK) throw Error(tail, "pair buffer smaller than the pair count; counts are valid");
}

// ------------------------------------------------------------------ fused batch join
// Units of instance i of a class occupy [off[i], off[i+1]) of the class's
// list: tag each with its instance (index into the batch's InstDesc array).
__global__ void k_unit_inst(const unsigned long long* __restrict__ off, uint32_t n_inst, const uint32_t* __restrict__ gidx,
                            uint32_t* __restrict__ unit_inst, unsigned long long total) {
  const unsigned long long t = (unsigned long long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= total) return;
  uint32_t lo = 0, hi = n_inst - 1;  // last instance whose first unit is <= t
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (off[mid] <= t) lo = mid; else hi = mid - 1;
  }
  unit_inst[t] = gidx[lo];
}

// Sorted packed pairs of global row ids -> local ids of their instance
// (row0 of the instance subtracted from both halves) in memory order (i, j).
__global__ void k_localize(unsigned long long* __restrict__ p, size_t np, const uint32_t* __restrict__ row0,
                           uint32_t n_inst) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= np) return;
  const unsigned long long v = p[t];
  const uint32_t gi = (uint32_t)(v >> 32), gj = (uint32_t)v;
  uint32_t lo = 0, hi = n_inst - 1;
  while (lo < hi) {
    const uint32_t mid = (lo + hi + 1) >> 1;
    if (row0[mid] <= gi) lo = mid; else hi = mid - 1;
  }
  const uint32_t r0 = row0[lo];
  p[t] = ((unsigned long long)(gj - r0) << 32) | (gi - r0);
}

// All instances of a batch in one pass of the join kernels.  Phase one
// builds every instance's index and work lists on worker streams
// (run_selfjoin with a BatchExport) into one batch arena.  Phase two, on the
// handle's stream and captured as one CUDA graph: per dimensionality class,
// the instances' unit lists are concatenated and tagged with their instance,
// one persistent CUDA-core launch and one persistent tensor-core launch drain
// all of them (each unit reads its instance's rows, bins and thresholds),
// and one band-decision launch finishes every instance.  Pairs carry global
// row ids; accepted pairs are counted per instance as they are staged.  The
// reference runs one process per dataset (script.sh:86-117); its nearest
// device-side idea is nodeByPoint4's atomic point queue (src/kernel.cu:912-989).
mistic_status run_batch_fused(mistic_handle h, const mistic_instance* inst, uint32_t m, const mistic_opts& o,
                              mistic_result* results, unsigned W, std::string* msg) {
  const auto wall0 = std::chrono::steady_clock::now();
  // ---- batch arena: bump allocation for the exported work lists
  std::vector<uint32_t> row0(m);
  size_t est = 64u << 20;
  {
    unsigned long long acc = 0;
    for (uint32_t i = 0; i < m; ++i) {
      row0[i] = (uint32_t)acc;
      acc += inst[i].n;
      const size_t esz = inst[i].dtype == MISTIC_F64 ? 8 : 4;
      est += inst[i].n * (((inst[i].d + 3) & ~3u) * 4 + 96 + (o.input_on_device ? 0 : inst[i].d * esz)) + 4096;
    }
    if (acc >= 0xffffffffull) return MISTIC_ERR_TOO_LARGE;  // global row ids are 32-bit
  }
  unsigned char* arena = (unsigned char*)h->arena.get("batch", est);
  const size_t arena_bytes = h->arena.bufs["batch"].bytes;
  size_t arena_used = 0;
  std::mutex amu;
  auto alloc = [&](size_t b) -> void* {
    std::lock_guard<std::mutex> g(amu);
    b = (b + 255) & ~(size_t)255;
    if (arena_used + b > arena_bytes) return nullptr;  // that instance is joined on its own instead
    void* p = arena + arena_used;
    arena_used += b;
    return p;
  };
  std::vector<BatchExport> ex(m);
  for (uint32_t i = 0; i < m; ++i) {
    ex[i].row0 = row0[i];
    ex[i].alloc = alloc;
  }
  // ---- phase one on the worker handles
  std::atomic<uint32_t> next{0};
  std::atomic<bool> stop{false};
  std::mutex mu;
  uint32_t err_i = UINT32_MAX;
  mistic_status err_s = MISTIC_OK;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < W; ++t) {
    th.emplace_back([&, t]() {
      mistic_handle w = h->workers[t];
      cudaSetDevice(h->device);
      for (;;) {
        const uint32_t i = next.fetch_add(1);
        if (i >= m || stop.load()) break;
        mistic_status s = MISTIC_OK;
        std::string em;
        try {
          run_selfjoin(w, inst[i].pts, inst[i].n, inst[i].d, inst[i].dtype, inst[i].k, inst[i].eps, &o, &results[i],
                       &ex[i]);
        } catch (const Error& e) {
          s = e.status;
          em = e.what();
        } catch (const std::exception& e) {
          s = MISTIC_ERR_INTERNAL;
          em = e.what();
        }
        if (s != MISTIC_OK) {
          std::lock_guard<std::mutex> g(mu);
          if (i < err_i) {
            err_i = i;
            err_s = s;
            *msg = em;
          }
          stop.store(true);
        }
      }
    });
  }
  for (auto& x : th) x.join();
  if (err_s != MISTIC_OK) return err_s;

  // ---- phase two: classes of exported instances by d
  std::vector<uint32_t> gl;  // exported instance -> batch index, ascending (so row0 ascends too)
  for (uint32_t i = 0; i < m; ++i)
    if (ex[i].exported) gl.push_back(i);
  if (gl.empty()) return MISTIC_OK;
  const uint32_t G = (uint32_t)gl.size();
  std::map<uint32_t, std::vector<uint32_t>> cls;  // d -> positions in gl
  for (uint32_t g = 0; g < G; ++g) cls[inst[gl[g]].d].push_back(g);
  unsigned long long tot_u = 0, tot_ut = 0, cand = 0, tot_n = 0;
  for (uint32_t g = 0; g < G; ++g) {
    tot_u += ex[gl[g]].n_units;
    tot_ut += ex[gl[g]].n_units_tc;
    cand += results[gl[g]].candidates;
    tot_n += inst[gl[g]].n;
  }
  const size_t nc = cls.size();
  // device tables, allocated before the capture
  InstDesc* d_desc = abuf<InstDesc>(h, "b_desc", G);
  uint32_t* d_row0 = abuf<uint32_t>(h, "b_row0", G);
  unsigned long long* d_ipairs = abuf<unsigned long long>(h, "b_ipairs", G);
  Unit* d_units = abuf<Unit>(h, "b_units", tot_u + 1);
  Unit* d_units_tc = abuf<Unit>(h, "b_units_tc", tot_ut + 1);
  uint32_t* d_uinst = abuf<uint32_t>(h, "b_uinst", tot_u + 1);
  uint32_t* d_uinst_tc = abuf<uint32_t>(h, "b_uinst_tc", tot_ut + 1);
  unsigned long long* d_off = abuf<unsigned long long>(h, "b_off", 2 * (G + nc) + 2);
  uint32_t* d_gidx = abuf<uint32_t>(h, "b_gidx", G + 1);
  JoinCounters* ctr = abuf<JoinCounters>(h, "b_ctr", 2);
  {
    std::vector<InstDesc> hd(G);
    std::vector<uint32_t> hr(G);
    for (uint32_t g = 0; g < G; ++g) {
      hd[g] = ex[gl[g]].desc;
      hr[g] = ex[gl[g]].desc.row0;
    }
    MCK(cudaMemcpyAsync(d_desc, hd.data(), G * sizeof(InstDesc), cudaMemcpyHostToDevice, h->stream));
    MCK(cudaMemcpyAsync(d_row0, hr.data(), G * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  }
  // per class: unit offsets (simt, tc) and the class's instance -> batch table
  struct Cls {
    uint32_t d, dpad32;
    int CH;
    unsigned long long u0, nu, t0, nt;  // ranges in the batch unit lists
    unsigned long long* off_u;          // device prefix of unit counts (n_inst + 1)
    unsigned long long* off_t;
    uint32_t* gidx;                     // device: class instance -> exported index
    uint32_t ninst;
    std::vector<uint32_t> members;
  };
  std::vector<Cls> C;
  {
    std::vector<unsigned long long> hoff;
    std::vector<uint32_t> hg;
    unsigned long long uu = 0, tt = 0;
    size_t offpos = 0, gpos = 0;
    for (auto& kv : cls) {
      Cls c;
      c.d = kv.first;
      c.members = kv.second;
      c.ninst = (uint32_t)kv.second.size();
      c.dpad32 = ex[gl[kv.second[0]]].dpad32;
      c.CH = ex[gl[kv.second[0]]].CH;
      c.u0 = uu;
      c.t0 = tt;
      c.off_u = d_off + offpos;
      c.off_t = d_off + offpos + c.ninst + 1;
      c.gidx = d_gidx + gpos;
      unsigned long long a = 0, b = 0;
      std::vector<unsigned long long> ou(c.ninst + 1), ot(c.ninst + 1);
      for (uint32_t j = 0; j < c.ninst; ++j) {
        ou[j] = a;
        ot[j] = b;
        a += ex[gl[kv.second[j]]].n_units;
        b += ex[gl[kv.second[j]]].n_units_tc;
        hg.push_back(kv.second[j]);
      }
      ou[c.ninst] = a;
      ot[c.ninst] = b;
      c.nu = a;
      c.nt = b;
      hoff.insert(hoff.end(), ou.begin(), ou.end());
      hoff.insert(hoff.end(), ot.begin(), ot.end());
      offpos += 2 * (c.ninst + 1);
      gpos += c.ninst;
      uu += a;
      tt += b;
      C.push_back(std::move(c));
    }
    MCK(cudaMemcpyAsync(d_off, hoff.data(), hoff.size() * sizeof(unsigned long long), cudaMemcpyHostToDevice,
                        h->stream));
    MCK(cudaMemcpyAsync(d_gidx, hg.data(), hg.size() * sizeof(uint32_t), cudaMemcpyHostToDevice, h->stream));
  }
  // pair list (when wanted) and band list
  const bool want_pairs = o.pairs != MISTIC_PAIRS_NONE;
  unsigned long long cap = 0;
  unsigned long long* pbuf = nullptr;
  if (want_pairs) {
    cap = std::max<unsigned long long>(1ull << 20, 16ull * tot_n);
    auto it = h->arena.bufs.find("b_pairs");
    if (it != h->arena.bufs.end()) cap = std::max<unsigned long long>(cap, it->second.bytes / 8);
  }
  unsigned long long bcap = std::max<unsigned long long>(1ull << 20, 2ull * tot_n);
  bcap = std::max<unsigned long long>(bcap, std::min<unsigned long long>(cand / 8192, 1ull << 30));
  {
    auto it = h->arena.bufs.find("b_band");
    if (it != h->arena.bufs.end()) bcap = std::max<unsigned long long>(bcap, it->second.bytes / 8);
    if (const char* e = getenv("MISTIC_BAND_CAP")) bcap = std::max<unsigned long long>(1, strtoull(e, nullptr, 10));
  }
  const bool use_graph = !(getenv("MISTIC_BATCH_GRAPH") && *getenv("MISTIC_BATCH_GRAPH") == '0');
  JoinCounters hc{};
  std::vector<unsigned long long> ipairs(G);
  float ms_fused = 0;
  bool complete = false;
  for (int attempt = 0; attempt < 3 && !complete; ++attempt) {
    if (want_pairs) pbuf = abuf<unsigned long long>(h, "b_pairs", cap);
    unsigned long long* band = abuf<unsigned long long>(h, "b_band", bcap);
    // ---- the fused pass: recorded into one CUDA graph (or issued directly)
    auto issue = [&]() {
      MCK(cudaMemsetAsync(ctr, 0, 2 * sizeof(JoinCounters), h->stream));
      MCK(cudaMemsetAsync(d_ipairs, 0, G * sizeof(unsigned long long), h->stream));
      for (const Cls& c : C) {
        unsigned long long pu = 0, pt = 0;
        for (uint32_t j = 0; j < c.ninst; ++j) {
          const BatchExport& e = ex[gl[c.members[j]]];
          if (e.n_units)
            MCK(cudaMemcpyAsync(d_units + c.u0 + pu, e.units, e.n_units * sizeof(Unit), cudaMemcpyDeviceToDevice,
                                h->stream));
          if (e.n_units_tc)
            MCK(cudaMemcpyAsync(d_units_tc + c.t0 + pt, e.units_tc, e.n_units_tc * sizeof(Unit),
                                cudaMemcpyDeviceToDevice, h->stream));
          pu += e.n_units;
          pt += e.n_units_tc;
        }
        if (c.nu) {
          k_unit_inst<<<(unsigned)((c.nu + 255) / 256), 256, 0, h->stream>>>(c.off_u, c.ninst, c.gidx,
                                                                            d_uinst + c.u0, c.nu);
          launched(h, "unit_inst");
        }
        if (c.nt) {
          k_unit_inst<<<(unsigned)((c.nt + 255) / 256), 256, 0, h->stream>>>(c.off_t, c.ninst, c.gidx,
                                                                            d_uinst_tc + c.t0, c.nt);
          launched(h, "unit_inst");
        }
      }
      for (const Cls& c : C) {
        JoinParams jp{};
        jp.units = d_units + c.u0;
        jp.n_units = c.nu;
        jp.dpad = c.dpad32;
        jp.d = c.d;
        jp.pairs = pbuf;
        jp.cap = cap;
        jp.band_list = band;
        jp.band_cap = bcap;
        jp.ctr = ctr;
        jp.insts = d_desc;
        jp.unit_inst = d_uinst + c.u0;
        jp.inst_row0 = d_row0;
        jp.n_inst = G;
        jp.inst_pairs = d_ipairs;
        // each launch drains its own list from the start
        MCK(cudaMemsetAsync(&ctr[0].next_unit, 0, sizeof(unsigned long long), h->stream));
        MCK(cudaMemsetAsync(&ctr[1].next_unit, 0, sizeof(unsigned long long), h->stream));
        join::run(h, false, c.CH, jp);
        if (c.nt) {
          TcParams tp{};
          tp.units = d_units_tc + c.t0;
          tp.n_units = c.nt;
          tp.ctr = ctr + 1;
          tp.unit_inst = d_uinst_tc + c.t0;
          tp.b = ex[gl[c.members[0]]].desc.tcb;  // per unit from its instance in the kernel
          tp.wait_limit = 2000000000ll;
          tp.prec = 0;
          join::run_tc(h, jp, tp);
        }
      }
      JoinParams jb{};
      jb.ctr = ctr;
      jb.pairs = pbuf;
      jb.cap = cap;
      jb.band_list = band;
      jb.band_cap = bcap;
      jb.insts = d_desc;
      jb.inst_row0 = d_row0;
      jb.n_inst = G;
      jb.inst_pairs = d_ipairs;
      join::run_band(h, jb);
    };
    MCK(cudaEventRecord(h->jev[0], h->stream));
    if (use_graph) {
      cudaGraph_t graph = nullptr;
      cudaGraphExec_t exec = nullptr;
      MCK(cudaStreamBeginCapture(h->stream, cudaStreamCaptureModeThreadLocal));
      try {
        issue();
      } catch (...) {
        cudaStreamEndCapture(h->stream, &graph);
        if (graph) cudaGraphDestroy(graph);
        cudaGetLastError();
        throw;
      }
      MCK(cudaStreamEndCapture(h->stream, &graph));
      const cudaError_t ie = cudaGraphInstantiate(&exec, graph, 0);
      cudaGraphDestroy(graph);
      MCK(ie);
      const cudaError_t le = cudaGraphLaunch(exec, h->stream);
      cudaGraphExecDestroy(exec);  // destruction waits for nothing: the launch is already queued
      MCK(le);
    } else {
      issue();
    }
    MCK(cudaEventRecord(h->jev[1], h->stream));
    MCK(cudaMemcpyAsync(&hc, ctr, sizeof hc, cudaMemcpyDeviceToHost, h->stream));
    MCK(cudaMemcpyAsync(ipairs.data(), d_ipairs, G * sizeof(unsigned long long), cudaMemcpyDeviceToHost, h->stream));
    MCK(cudaStreamSynchronize(h->stream));
    MCK(cudaEventElapsedTime(&ms_fused, h->jev[0], h->jev[1]));
    JoinCounters tcc{};
    MCK(cudaMemcpy(&tcc, ctr + 1, sizeof tcc, cudaMemcpyDeviceToHost));
    if (hc.error || tcc.error) throw Error(MISTIC_ERR_TIMEOUT, "a tensor-core tile wait timed out");
    if (hc.band_n > bcap) {
      bcap = hc.band_n + hc.band_n / 4;
      continue;
    }
    if (want_pairs && hc.pairs > cap) {
      cap = hc.pairs + hc.pairs / 8;
      continue;
    }
    complete = true;
  }
  if (!complete) throw Error(MISTIC_ERR_INTERNAL, "the fused batch join still overflowed after its last pass");
  // ---- per-instance results
  std::vector<unsigned long long> pstart(G + 1, 0);
  if (want_pairs && hc.pairs) {
    uint64_t* pk[2] = {(uint64_t*)pbuf, abuf<uint64_t>(h, "b_pairs_tmp", hc.pairs)};
    uint32_t* pv[2] = {nullptr, nullptr};
    const int c = radix_sort_u64(h, pk, pv, false, false, hc.pairs, 32 + bit_length(tot_n ? row0.back() + inst[m - 1].n : 1));
    unsigned long long* sorted = (unsigned long long*)pk[c];
    for (uint32_t g = 0; g < G; ++g) pstart[g + 1] = pstart[g] + ipairs[g];
    if (pstart[G] != hc.pairs) throw Error(MISTIC_ERR_INTERNAL, "per-instance pair counts do not add up");
    k_localize<<<(unsigned)((hc.pairs + 255) / 256), 256, 0, h->stream>>>(sorted, hc.pairs, d_row0, G);
    launched(h, "localize");
    for (uint32_t g = 0; g < G; ++g) {
      mistic_result& r = results[gl[g]];
      const unsigned long long np = ipairs[g];
      r.pairs_len = np;
      if (o.pairs == MISTIC_PAIRS_HOST) {
        // each instance's slice of the sorted list straight into its own
        // pinned block (a staging copy through one pageable array cost two
        // passes over the host memory of every pair)
        uint32_t* hp = (uint32_t*)pinned_cache().acquire(std::max<size_t>(1, np * 8));
        if (!hp) hp = (uint32_t*)malloc(std::max<size_t>(1, np * 8));
        if (!hp) throw Error(MISTIC_ERR_OUT_OF_MEMORY, "host pair buffer");
        r.pairs = hp;
        r.pairs_on_device = 0;
        r._owner = hp;
        if (np) MCK(cudaMemcpyAsync(hp, sorted + pstart[g], np * 8, cudaMemcpyDeviceToHost, h->stream));
      } else {
        void* dp = nullptr;
        MCK(cudaMalloc(&dp, std::max<size_t>(8, np * 8)));
        MCK(cudaMemcpyAsync(dp, sorted + pstart[g], np * 8, cudaMemcpyDeviceToDevice, h->stream));
        r.pairs = (uint32_t*)dp;
        r.pairs_on_device = 1;
        r._owner = dp;
      }
    }
    MCK(cudaStreamSynchronize(h->stream));
  }
  const double wall = std::chrono::duration<double, std::milli>(std::chrono::steady_clock::now() - wall0).count();
  for (uint32_t g = 0; g < G; ++g) {
    mistic_result& r = results[gl[g]];
    r.pairs_ij = ipairs[g];
    r.pairs_ordered_incl_self = 2 * ipairs[g] + r.n;
    r.ms_join = ms_fused;  // the fused join pass is shared by all instances of the batch
    r.ms_wall = wall;
    r.ulp_ambiguous = 0;
    r.band_pairs = 0;
  }
  return MISTIC_OK;
}

}  // namespace

// Directed edges of the neighbour table: both orientations of every pair
// plus every point's self edge, packed (src << 32 | dst).
__global__ void k_csr_edges(const unsigned long long* __restrict__ pairs, size_t np, size_t n,
                            unsigned long long* __restrict__ e) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t < np) {
    const unsigned long long v = pairs[t];
    e[2 * t] = v;
    e[2 * t + 1] = (v << 32) | (v >> 32);
  } else if (t < np + n) {
    const unsigned long long p = t - np;
    e[2 * np + p] = (p << 32) | p;
  }
}

// Sorted edges -> neighbour ids and row offsets (every row has its self edge,
// so every row starts somewhere).
__global__ void k_csr_split(const unsigned long long* __restrict__ e, size_t E, uint32_t* __restrict__ nbrs,
                            unsigned long long* __restrict__ offs, size_t n) {
  const size_t t = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= E) return;
  const unsigned long long v = e[t];
  nbrs[t] = (uint32_t)v;
  const unsigned long long src = v >> 32;
  if (t == 0 || (e[t - 1] >> 32) != src) offs[src] = t;
  if (t == 0) offs[n] = E;
}

void csr_edges(mistic_handle_s* h, const unsigned long long* pairs, size_t np, size_t n, unsigned long long* e) {
  const size_t tot = np + n;
  k_csr_edges<<<(unsigned)((tot + 255) / 256), 256, 0, h->stream>>>(pairs, np, n, e);
  launched(h, "csr_edges");
}

void csr_split(mistic_handle_s* h, const unsigned long long* e, size_t E, uint32_t* nbrs, unsigned long long* offs,
               size_t n) {
  k_csr_split<<<(unsigned)((E + 255) / 256), 256, 0, h->stream>>>(e, E, nbrs, offs, n);
  launched(h, "csr_split");
}

__global__ void k_pairs_to_ij(unsigned long long* p, size_t n) {
  const size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const unsigned long long v = p[i];
  // packed (i << 32 | j) -> memory order (i, j) as two uint32
  p[i] = (v >> 32) | (v << 32);
}

void pairs_to_ij(mistic_handle_s* h, unsigned long long* p, size_t n) {
  if (!n) return;
  k_pairs_to_ij<<<(unsigned)((n + 255) / 256), 256, 0, h->stream>>>(p, n);
  launched(h, "pairs_to_ij");
}

}  // namespace mistic

// ====================================================================== C ABI
using mistic::Error;

static mistic_status fail(mistic_handle h, mistic_status s, const char* msg) {
  if (h) h->last_error = msg;
  return s;
}

#define MISTIC_GUARD(h, body)                                                   \
  try {                                                                         \
    body;                                                                       \
    return MISTIC_OK;                                                           \
  } catch (const Error& e) {                                                    \
    return fail(h, e.status, e.what());                                         \
  } catch (const std::bad_alloc&) {                                             \
    return fail(h, MISTIC_ERR_OUT_OF_MEMORY, "host allocation failed");         \
  } catch (const std::exception& e) {                                           \
    return fail(h, MISTIC_ERR_INTERNAL, e.what());                              \
  } catch (...) {                                                               \
    return fail(h, MISTIC_ERR_INTERNAL, "unknown failure");                     \
  }

extern "C" {

int mistic_abi_version(void) { return MISTIC_ABI_VERSION; }

void mistic_opts_init(mistic_opts* o) {
  if (!o) return;
  memset(o, 0, sizeof(*o));
  o->struct_size = sizeof(mistic_opts);
  o->mode = MISTIC_MODE_AUTO;
  o->rp_mode = MISTIC_RP_PCA;
  o->seed = 0;
  o->pairs = MISTIC_PAIRS_NONE;
  o->check_finite = 1;
  o->timing = 1;
}

mistic_status mistic_create(mistic_handle* out, int device, void* stream) {
  if (!out) return MISTIC_ERR_INVALID_ARG;
  *out = nullptr;
  int ndev = 0;
  if (cudaGetDeviceCount(&ndev) != cudaSuccess || ndev == 0) {
    cudaGetLastError();
    return MISTIC_ERR_NO_DEVICE;
  }
  if (device < 0 || device >= ndev) return MISTIC_ERR_INVALID_ARG;
  mistic_handle h = new (std::nothrow) mistic_handle_s();
  if (!h) return MISTIC_ERR_OUT_OF_MEMORY;
  try {
    MCK(cudaSetDevice(device));
    cudaDeviceProp p;
    MCK(cudaGetDeviceProperties(&p, device));
    if (p.major < 10) throw Error(MISTIC_ERR_NO_DEVICE, "libmistic is built for sm_103a (Blackwell)");
    h->device = device;
    h->sms = p.multiProcessorCount;
    {
      int pma = 0, hpt = 0;
      cudaDeviceGetAttribute(&pma, cudaDevAttrPageableMemoryAccess, device);
      cudaDeviceGetAttribute(&hpt, cudaDevAttrPageableMemoryAccessUsesHostPageTables, device);
      cudaGetLastError();
      const char* e = getenv("MISTIC_HOST_READS");  // 0: staging ring / plain copies only
      h->host_reads = pma && hpt && !(e && *e == '0');
      const char* e2 = getenv("MISTIC_HOST_PAIRS");  // 0: host pair lists by a copy after the join
      h->host_pairs = pma && hpt && !(e2 && *e2 == '0');
    }
    if (stream) {
      h->stream = (cudaStream_t)stream;
    } else {
      MCK(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
      h->own_stream = true;
    }
    h->arena.stream = h->stream;
    for (auto& e : h->ev) MCK(cudaEventCreate(&e));
    for (auto& e : h->jev) MCK(cudaEventCreate(&e));
  } catch (const Error& e) {
    mistic_status s = e.status;
    if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
    delete h;
    return s;
  }
  *out = h;
  return MISTIC_OK;
}

mistic_status mistic_destroy(mistic_handle h) {
  if (!h) return MISTIC_ERR_INVALID_ARG;
  cudaSetDevice(h->device);
  cudaStreamSynchronize(h->stream);
  h->arena.release_all();
  if (h->pinned) cudaFreeHost(h->pinned);
  if (h->stage) cudaFreeHost(h->stage);
  for (auto& e : h->stage_ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : h->ev)
    if (e) cudaEventDestroy(e);
  for (auto& e : h->jev)
    if (e) cudaEventDestroy(e);
  for (auto& e : h->hr_ev)
    if (e) cudaEventDestroy(e);
  if (h->own_stream) cudaStreamDestroy(h->stream);
  for (mistic_handle w : h->workers) mistic_destroy(w);
  if (h->batch_ev) cudaEventDestroy(h->batch_ev);
  delete h;
  return MISTIC_OK;
}

mistic_status mistic_bruteforce_rows(mistic_handle h, const void* pts, uint64_t n, uint32_t d, mistic_dtype dtype,
                                    double eps, uint64_t row0, uint64_t row1, int input_on_device,
                                    uint32_t* counts) {
  MISTIC_GUARD(h, {
    mistic::check_handle(h);
    if (d == 0 || (n > 0 && !pts) || !counts || row0 > row1 || row1 > n)
      throw mistic::Error(MISTIC_ERR_INVALID_ARG, "bad brute-force arguments");
    if (dtype != MISTIC_F64 && dtype != MISTIC_F32) throw mistic::Error(MISTIC_ERR_INVALID_ARG, "bad dtype");
    if (!(eps >= 0.0) || !std::isfinite(eps)) throw mistic::Error(MISTIC_ERR_INVALID_ARG, "eps must be finite and >= 0");
    if (row1 == row0) return MISTIC_OK;
    const size_t esz = dtype == MISTIC_F64 ? 8 : 4;
    const void* x = pts;
    if (!input_on_device) {
      void* dx = h->arena.get("bf_raw", n * d * esz);
      mistic::h2d(h, dx, pts, n * d * esz);
      x = dx;
    }
    uint32_t* dc = (uint32_t*)h->arena.get("bf_counts", (row1 - row0) * sizeof(uint32_t));
    mistic::bruteforce_rows(h, x, dtype, n, d, eps * eps, row0, row1, dc);
    mistic::d2h(h, counts, dc, (row1 - row0) * sizeof(uint32_t));
  });
}

mistic_status mistic_selfjoin(mistic_handle h, const void* pts, uint64_t n, uint32_t d, mistic_dtype dtype,
                              uint32_t k, double eps, const mistic_opts* opts, mistic_result* result) {
  MISTIC_GUARD(h, mistic::run_selfjoin(h, pts, n, d, dtype, k, eps, opts, result));
}

// Instances run concurrently on a pool of worker handles (own streams, own
// buffers, created once per handle), driven by host threads that take the
// next instance from an atomic index: small instances are bound by launch
// and read-back latency, which the streams overlap.  MISTIC_BATCH_STREAMS
// sets the pool size (default min(8, host threads); 1 = one after another
// on this handle).  A caller pair buffer forces the serial order (one
// buffer cannot hold concurrent lists).  On a failure the lowest failing
// instance's status and message are returned; instances not run keep a
// zeroed result.
mistic_status mistic_batch_selfjoin(mistic_handle h, const mistic_instance* inst, uint32_t m,
                                    const mistic_opts* opts, mistic_result* results) {
  if (!h || (m > 0 && (!inst || !results))) return fail(h, MISTIC_ERR_INVALID_ARG, "null argument");
  unsigned want = std::max(1u, std::min(8u, std::thread::hardware_concurrency()));
  if (const char* e = getenv("MISTIC_BATCH_STREAMS")) want = (unsigned)std::max(1l, strtol(e, nullptr, 10));
  const unsigned W = std::min<unsigned>(want, m);
  mistic_opts o;
  mistic_opts_init(&o);
  if (opts) {
    if (opts->struct_size != sizeof(mistic_opts))
      return fail(h, MISTIC_ERR_INVALID_ARG, "mistic_opts.struct_size mismatch (call mistic_opts_init)");
    o = *opts;
  }
  // fused: every instance's units drained by shared persistent launches
  // (run_batch_fused); MISTIC_BATCH_FUSED=0 keeps one pipeline per instance
  const char* fz = getenv("MISTIC_BATCH_FUSED");
  const bool fused = m > 1 && !(fz && *fz == '0') && !o.pair_buffer && o.csr == MISTIC_PAIRS_NONE &&
                     (o.mode == MISTIC_MODE_AUTO || o.mode == MISTIC_MODE_BF16 || o.mode == MISTIC_MODE_FP32);
  if (!fused && (W <= 1 || o.pair_buffer)) {
    for (uint32_t i = 0; i < m; ++i) {
      mistic_status s = mistic_selfjoin(h, inst[i].pts, inst[i].n, inst[i].d, inst[i].dtype, inst[i].k,
                                        inst[i].eps, opts, &results[i]);
      if (s != MISTIC_OK) return s;
    }
    return MISTIC_OK;
  }
  memset(results, 0, sizeof(mistic_result) * m);
  try {
    MCK(cudaSetDevice(h->device));
    while (h->workers.size() < W) {
      mistic_handle w = nullptr;
      const mistic_status s = mistic_create(&w, h->device, nullptr);
      if (s != MISTIC_OK) throw Error(s, "batch worker handle");
      h->workers.push_back(w);
    }
    if (!h->batch_ev) MCK(cudaEventCreateWithFlags(&h->batch_ev, cudaEventDisableTiming));
    MCK(cudaEventRecord(h->batch_ev, h->stream));  // inputs produced on the caller's stream
    for (unsigned t = 0; t < W; ++t) MCK(cudaStreamWaitEvent(h->workers[t]->stream, h->batch_ev, 0));
  } catch (const Error& e) {
    return fail(h, e.status, e.what());
  }
  if (fused) {
    std::string msg;
    mistic_status st = MISTIC_OK;
    try {
      st = mistic::run_batch_fused(h, inst, m, o, results, std::max(1u, W), &msg);
    } catch (const Error& e) {
      st = e.status;
      msg = e.what();
    } catch (const std::bad_alloc&) {
      st = MISTIC_ERR_OUT_OF_MEMORY;
      msg = "host allocation failed";
    } catch (const std::exception& e) {
      st = MISTIC_ERR_INTERNAL;
      msg = e.what();
    }
    if (st != MISTIC_OK) {
      // copies into the results' blocks may still be in flight: let them
      // land before the blocks go back to the pinned cache
      cudaStreamSynchronize(h->stream);
      cudaGetLastError();
      for (uint32_t i = 0; i < m; ++i) mistic_result_free(&results[i]);
      return fail(h, st, msg.empty() ? mistic_strerror(st) : msg.c_str());
    }
    return MISTIC_OK;
  }
  std::atomic<uint32_t> next{0};
  std::atomic<bool> stop{false};
  std::mutex mu;
  uint32_t err_i = UINT32_MAX;
  mistic_status err_s = MISTIC_OK;
  std::string err_msg;
  std::vector<std::thread> th;
  for (unsigned t = 0; t < W; ++t) {
    th.emplace_back([&, t]() {
      mistic_handle w = h->workers[t];
      cudaSetDevice(h->device);
      for (;;) {
        const uint32_t i = next.fetch_add(1);
        if (i >= m || stop.load()) break;
        const mistic_status s = mistic_selfjoin(w, inst[i].pts, inst[i].n, inst[i].d, inst[i].dtype, inst[i].k,
                                                inst[i].eps, opts, &results[i]);
        if (s != MISTIC_OK) {
          std::lock_guard<std::mutex> g(mu);
          if (i < err_i) {
            err_i = i;
            err_s = s;
            err_msg = w->last_error;
          }
          stop.store(true);
        }
      }
    });
  }
  for (auto& x : th) x.join();
  if (err_s != MISTIC_OK) return fail(h, err_s, err_msg.c_str());
  return MISTIC_OK;
}

mistic_status mistic_read_points(const char* path, uint32_t d, mistic_dtype dtype, void** out_pts,
                                 uint64_t* out_n) {
  if (!path || !out_pts || !out_n || d == 0) return MISTIC_ERR_INVALID_ARG;
  if (dtype != MISTIC_F64 && dtype != MISTIC_F32) return MISTIC_ERR_INVALID_ARG;
  *out_pts = nullptr;
  *out_n = 0;
  std::ifstream f(path, std::ios::in | std::ios::binary);
  if (!f) return MISTIC_ERR_IO;
  f.seekg(0, std::ios::end);
  const std::streamoff size = f.tellg();
  if (size < 0) return MISTIC_ERR_IO;
  f.seekg(0, std::ios::beg);
  const size_t esz = dtype == MISTIC_F64 ? 8 : 4;
  const uint64_t n = (uint64_t)size / esz / d;
  void* buf = malloc(std::max<size_t>(1, (size_t)(n * d * esz)));
  if (!buf) return MISTIC_ERR_OUT_OF_MEMORY;
  if (n && !f.read((char*)buf, (std::streamsize)(n * d * esz))) {
    free(buf);
    return MISTIC_ERR_IO;
  }
  *out_pts = buf;
  *out_n = n;
  return MISTIC_OK;
}

void mistic_free_host(void* p) { free(p); }

void mistic_result_free(mistic_result* r) {
  if (!r) return;
  if (r->pairs && r->_owner) {
    if (r->pairs_on_device)
      cudaFree(r->pairs);
    else if (!mistic::pinned_cache().release(r->pairs))
      free(r->pairs);
  }
  r->pairs = nullptr;
  r->_owner = nullptr;
  if (r->csr_on_device) {
    if (r->csr_offsets) cudaFree(r->csr_offsets);
    if (r->csr_nbrs) cudaFree(r->csr_nbrs);
  } else {
    free(r->csr_offsets);
    free(r->csr_nbrs);
  }
  r->csr_offsets = nullptr;
  r->csr_nbrs = nullptr;
  r->pairs_len = 0;
}

const char* mistic_strerror(mistic_status s) {
  switch (s) {
    case MISTIC_OK: return "ok";
    case MISTIC_ERR_INVALID_ARG: return "invalid argument";
    case MISTIC_ERR_CUDA: return "CUDA runtime error";
    case MISTIC_ERR_OUT_OF_MEMORY: return "out of memory";
    case MISTIC_ERR_TOO_LARGE: return "problem too large";
    case MISTIC_ERR_NOT_FINITE: return "non-finite input coordinate";
    case MISTIC_ERR_PAIR_OVERFLOW: return "pair buffer too small";
    case MISTIC_ERR_TIMEOUT: return "device wait timed out";
    case MISTIC_ERR_NO_DEVICE: return "no suitable CUDA device";
    case MISTIC_ERR_IO: return "I/O error";
    case MISTIC_ERR_INTERNAL: return "internal error";
  }
  return "unknown status";
}

const char* mistic_last_error(mistic_handle h) { return h ? h->last_error.c_str() : "null handle"; }

}  // extern "C"
