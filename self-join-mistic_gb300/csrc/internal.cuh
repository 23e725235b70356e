// Internal declarations shared by the libmistic translation units.
// Nothing here crosses the C ABI (include/mistic.h).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include <algorithm>
#include <map>
#include <mutex>
#include <stdexcept>
#include <string>
#include <vector>

#include "../../include/mistic.h"

namespace mistic {

constexpr unsigned FULL_MASK = 0xffffffffu;
constexpr int MAX_K = 16;        // reference points per bin key
constexpr int KEY_BITS_MAX = 63; // packed key budget (one spare bit keeps range ends in u64)
constexpr uint32_t MAX_D = 4096; // dimensionality limit of the join kernels

// Error carried from deep inside the pipeline to the C ABI boundary, where it
// becomes a mistic_status plus the handle's last-error text.
struct Error : std::runtime_error {
  mistic_status status;
  Error(mistic_status s, const std::string& m) : std::runtime_error(m), status(s) {}
};

[[noreturn]] void throw_cuda(cudaError_t e, const char* what, const char* file, int line);

#define MCK(call)                                                   \
  do {                                                              \
    cudaError_t e__ = (call);                                       \
    if (e__ != cudaSuccess) ::mistic::throw_cuda(e__, #call, __FILE__, __LINE__); \
  } while (0)

// Device buffers owned by a handle, grown on demand and reused across calls
// (the reference allocates everything per call, src/launcher.cu:3259-3349).
struct Arena {
  struct Buf {
    void* p = nullptr;
    size_t bytes = 0;
  };
  std::map<std::string, Buf> bufs;
  cudaStream_t stream = nullptr;  // work using the buffers; drained before a regrow
  void* get(const std::string& name, size_t bytes);
  void release_all();
};

// Key layout of the packed bin key: reference point j occupies `bits[j]`
// bits at `shift[j]`; reference point 0 is the most significant field, so
// numeric order of the packed key is lexicographic order of the key vector.
struct KeyLayout {
  int k;
  int total_bits;
  int bits[MAX_K];
  int shift[MAX_K];
  int32_t minkey[MAX_K];  // subtracted before packing
  uint32_t maxkey[MAX_K]; // largest stored field value (after subtraction)
};

// One join work unit: a chunk of up to `CH` points of home bin `h` against
// the neighbour bins nbr[s0 .. s1) (all of index >= h).
struct Unit {
  uint32_t h;
  uint32_t chunk;
  uint32_t s0;
  uint32_t s1;
};

// Counters the join kernels accumulate on the device.
struct JoinCounters {
  unsigned long long pairs;      // accepted unordered pairs
  unsigned long long band;       // pairs re-decided in FP64
  unsigned long long ambiguous;  // FP64 value within 4 ulp of eps2
  unsigned long long next_unit;  // work-queue cursor
  unsigned long long error;      // non-zero: a bounded device wait gave up
  unsigned long long tiles;      // tensor-core tiles evaluated
  unsigned long long cells;      // sum over those tiles of home rows x candidate columns
  unsigned long long band_n;     // candidate pairs appended to the band list (decided afterwards in FP64)
  unsigned long long stop;       // pair ring: a list was full; no unit is claimed after it
  unsigned long long def_n;      // pair ring: units deferred in this pass
  unsigned long long prof[24];   // role cycle breakdown when TcParams.prof is set
};

// Key packing: field f = floor((D[i*kstride + col[f]] - dmin[f]) / w[f]),
// clamped to [0, maxkey[f]], stored at bit `shift[f]`.
struct PackParams {
  int k;
  int kstride;
  int col[MAX_K];
  double dmin[MAX_K];
  double w[MAX_K];
  uint32_t maxkey[MAX_K];
  int shift[MAX_K];
};

// Neighbour enumeration: the same field layout, plus the unit split sizes.
struct EnumParams {
  int k;
  int shift[MAX_K];
  uint32_t maxkey[MAX_K];
  uint32_t seg_cap;     // candidate points per neighbour segment (CUDA-core units)
  uint32_t seg_cap_tc;  // the same for tensor-core units
  uint32_t chunk;    // home points per CUDA-core unit
  uint32_t tc_min;   // home bins with at least this many points get tensor-core units (0: none)
  uint32_t tc_chunk; // home points per tensor-core unit
  uint32_t sample;   // > 1: only home points of sampled 512-point groups (mistic_opts.home_sample)
  // prefix table over the first p key fields (p = 0: none): ptab[v] = first
  // bin whose fields 0 .. p-1, as sum_j field_j * stride[j], are >= v
  int p;
  uint32_t stride[MAX_K];
  const uint32_t* ptab;
};

// FP32 constants of a tensor-core join's per-column error bound (see
// column_threshold in tc_common.cuh).
struct TcBound {
  float eps2_lo, eps2_hi;  // fl32 bounds of eps2/(1+g64), eps2/(1-g64)
  float kappa;             // relative MMA + norm error per (|a'|+|q'|)^2
  float ginf;              // norm inflation 1/(1-g_d)
  float uR2;               // 2uR (global centring error)
  float u1;                // u(1+u)
  float Dp;                // 1.1 sqrt(eps2)
  float cap;               // 0.1 eps2: larger bounds re-decide the whole column in FP64
  float margin;            // small positive slack that makes D' >= 0 a strict reject
};

// One instance of a fused batch join (mistic_batch_selfjoin): its sorted
// rows, bins and neighbour list, and its thresholds.  Join kernels given
// JoinParams.insts take each unit's instance from unit_inst and read these
// in place of the single-instance fields; ids are global (row0 + the
// instance's own row id), so pairs of different instances never collide.
struct InstDesc {
  const uint32_t* bstart;
  const uint32_t* nbr;
  const uint32_t* ids;
  const void* xs;      // sorted FP32 rows, stride dpad of the launch
  const void* raw;     // the instance's rows as given (device), for the FP64 decisions
  uint32_t d, raw_f32;
  uint32_t row0;       // first global row id of the instance
  float t_lo, t_hi;    // FP32 filter
  double eps2, amb;
  TcBound tcb;         // tensor-core bound
};

struct JoinParams {
  const Unit* units;
  unsigned long long n_units;
  const uint32_t* bstart;
  const uint32_t* nbr;
  const uint32_t* ids;
  const void* xs;       // sorted rows: float (FP32 mode) or double (FP64 mode), stride dpad
  uint32_t dpad;
  const void* raw;      // caller's rows (device), indexed by original id, for FP64 re-decision
  int raw_f32;
  uint32_t d;
  float t_lo, t_hi;     // FP32 mode: accept at or below t_lo, re-decide in (t_lo, t_hi]
  double eps2;          // fl(ε*ε)
  double amb;           // 4 ulp(eps2)
  unsigned long long* pairs;  // packed (i << 32 | j), i < j; null when counting only
  unsigned long long cap;
  int pairs_ij;               // non-zero: pairs are stored in memory order (i, j) instead (pair_ij)
  unsigned long long* band_list;  // packed (i << 32 | j) original ids whose fast value is inside the error band
  unsigned long long band_cap;
  JoinCounters* ctr;
  // fused batch joins only (null otherwise)
  const InstDesc* insts;             // per instance
  const uint32_t* unit_inst;         // instance of each unit of `units`
  const uint32_t* inst_row0;         // insts[i].row0, ascending (band decisions find a pair's instance)
  uint32_t n_inst;
  unsigned long long* inst_pairs;    // accepted pairs per instance
  // streamed pair ring only (mistic_opts.ring_capacity; `ring` 0 otherwise).
  // A launch claims the units def_in[0 .. n_def_in) (deferred by the last
  // pass), then main_start, main_start + 1, ... of its own list; unit u of
  // the CUDA-core list has tag u, unit u of the tensor-core list tag
  // n_units + u (tag_base_tc).
  int ring;
  uint32_t* pair_tags;               // unit tag of each pair-ring entry
  uint32_t* band_tags;               // unit tag of each band-list entry
  uint32_t* deferred;                // per tag: 1 once deferred in this pass
  uint32_t* def_out;                 // tags deferred in this pass (count in ctr->def_n)
  const uint32_t* def_in;            // CUDA-core list: units to run first (local indices)
  uint32_t n_def_in;
  unsigned long long main_start;     // CUDA-core list: first unit not yet claimed
  uint32_t tag_base_tc;
  unsigned long long band0, band1;   // band decisions of band_list[band0 .. band1) (pair ring)
  uint32_t grid_cap;                 // pair ring: at most this many blocks (0: the persistent grid)
  unsigned long long claim_cap;      // pair ring: claim indices from this one on take no unit (0: no cap)
  // FP32 pre-decision of band pairs (null inv: every band pair goes to FP64):
  // rows xf32[inv[id]] (sorted FP32 rows, stride dpad32) filtered with the
  // FP32 filter's thresholds t_lo / t_hi before the FP64 predicate
  const uint32_t* inv;
  const float* xf32;
  uint32_t dpad32;
};

// Tensor-core join: FP32 constants of the per-row error bound (see join_tc.cu).
struct TcParams {
  const Unit* units;
  unsigned long long n_units;
  JoinCounters* ctr;  // separate cursor from the CUDA-core join
  const uint32_t* unit_inst;  // fused batch joins: instance of each unit (JoinParams.insts), else null
  const uint32_t* def_in;     // pair ring: units to run first (local indices of `units`)
  uint32_t n_def_in;
  unsigned long long main_start;  // pair ring: first unit of `units` not yet claimed
  uint32_t grid_cap;          // pair ring: at most this many CTAs (0: one per SM)
  unsigned long long claim_cap;  // pair ring: claim indices from this one on take no unit (0: no cap)
  TcBound b;               // per-column bound constants (per instance in fused batch joins)
  long long wait_limit;    // nanoseconds before a barrier wait gives up
  int stall_test;          // failure-detection test: the MMA warp never signals (waits run out)
  int prof;                // record per-role wait/total cycles into ctr->prof (diagnostics)
  // long-row kernel (join_tcw.cu) only: prepared sorted rows and their norms
  int prec;                // operand precision: 0 split bf16, 1 single bf16, 2 tf32
  const void* xh;          // bf16 hi parts (prec 0, 1) or tf32-rounded FP32 rows (prec 2), n_rows x kd
  const void* xl;          // bf16 lo parts (prec 0), same layout
  const float* xn;         // FP32 |x|^2 of the sorted rows
  uint32_t kd;             // d rounded up to the stage's K
  uint64_t n_rows;         // rows of xh / xl
};

struct Timer {
  cudaEvent_t ev[24];
  int used = 0;
};

}  // namespace mistic

struct mistic_handle_s {
  int device = 0;
  cudaStream_t stream = nullptr;
  bool own_stream = false;
  int sms = 0;
  std::string last_error;
  mistic::Arena arena;
  void* pinned = nullptr;  // small pinned block for scalar read-backs
  size_t pinned_bytes = 0;
  // pinned staging ring for large host inputs (mistic::h2d): kStageSlots
  // slots of kStageSlotBytes, each with the event of its last DMA
  void* stage = nullptr;
  cudaEvent_t stage_ev[16] = {};
  cudaEvent_t ev[16] = {};
  cudaEvent_t jev[4] = {};  // around the two join kernels
  uint32_t launches = 0;
  bool host_reads = false;  // kernels may read pageable host memory (coherent CPU-GPU link, host page tables)
  // large host-read copies (mistic::h2d): events around the last one and its
  // size (0: none to check), and the large copies left to take through the
  // staging ring after one that ran slower than the ring
  cudaEvent_t hr_ev[2] = {};
  size_t hr_bytes = 0;
  uint32_t hr_skip = 0;
  bool host_pairs = false;  // join kernels may write host pair lists into pinned host memory (same link)
  unsigned long long host_pair_cap = 0;  // largest such host pair list so far (pairs)
  std::vector<mistic_handle_s*> workers;  // batch workers: own streams, same device (created on demand)
  cudaEvent_t batch_ev = nullptr;         // orders the workers' streams after this handle's stream
};

namespace mistic {

// Records a kernel launch for the result's kernel_launches counter and
// checks the launch status.
void launched(mistic_handle_s* h, const char* what);

// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum less the kernel's static shared memory, once per kernel and
// process.  The limit is a per-function setting; setting it to the size of
// each launch would let concurrent callers (batch worker threads) lower it
// under another thread's launch.
void allow_max_dyn_smem_impl(const void* kern);
template <class K>
void allow_max_dyn_smem(K kern) {
  allow_max_dyn_smem_impl(reinterpret_cast<const void*>(kern));
}

// ---- scan.cu
template <class T>
void exclusive_scan(mistic_handle_s* h, const T* in, T* out, size_t n, T* total_dev);
size_t scan_partials_count(size_t n);

// ---- sort.cu: LSD radix sort of 64-bit keys over the low `bits` bits with
// an optional 32-bit payload.  If vals_in is null the payload is the input
// position.  Returns which buffer (0/1) holds the result.
int radix_sort_u64(mistic_handle_s* h, uint64_t* keys[2], uint32_t* vals[2],
                   bool has_vals, bool iota_vals, size_t n, int bits);

// ---- index.cu
namespace idx {
void colstats(mistic_handle_s*, const void* x, mistic_dtype, size_t n, uint32_t d, double* part,
              uint32_t nparts, double* out, unsigned* nonfinite);
void sample_cov(mistic_handle_s*, const void* x, mistic_dtype, size_t n, uint32_t d, uint32_t S,
                double* sbuf, const double* mu, double* part, double* cov);
void rp_dist(mistic_handle_s*, const void* x, mistic_dtype, size_t n, uint32_t d, const double* rps,
             int k, double* D, double* part, uint32_t nparts, double* mm);
void pack_keys(mistic_handle_s*, const double* D, size_t n, const PackParams&, uint64_t* keys);
void iota(mistic_handle_s*, uint32_t* v, size_t n);
void bins(mistic_handle_s*, const uint64_t* keys, size_t n, uint32_t* flags, uint32_t* nbins_dev,
          uint32_t* bstart, uint64_t* bkey);
void gather(mistic_handle_s*, const void* x, mistic_dtype, size_t n, uint32_t d, const uint32_t* perm,
            const double* center, uint32_t dpad32, float* xf, uint32_t dpad64, double* xd,
            uint32_t* ids, double* norm_part, double* rmax);
// prefix table of the enumeration (EnumParams p, stride, shift): entries + 1
// values into ptab
void prefix_table(mistic_handle_s*, const uint64_t* bkey, uint32_t m, const EnumParams&, uint32_t* ptab,
                  uint32_t entries);
void enumerate(mistic_handle_s*, const uint64_t* bkey, const uint32_t* bstart, uint32_t m,
               const EnumParams&, uint32_t* nbr_cnt, uint32_t* unit_cnt, uint32_t* unit_cnt_tc,
               unsigned long long* cand, const uint32_t* nbr_off, const uint32_t* unit_off,
               const uint32_t* unit_off_tc, uint32_t* nbr, Unit* units, Unit* units_tc, bool fill);
// points per log2 bin-size class (32 classes) into hist
void bin_hist(mistic_handle_s*, const uint32_t* bstart, uint32_t m, unsigned long long* hist);
// 64-bit totals of the enumeration's three per-bin count arrays into tot[3]
void count_totals(mistic_handle_s*, const uint32_t* nbr_cnt, const uint32_t* unit_cnt, const uint32_t* unit_cnt_tc,
                  uint32_t m, unsigned long long* tot);
}  // namespace idx

// ---- mistic.cu: FP32 filter thresholds (accept at or below t_lo, re-decide
// in FP64 above it up to t_hi) for dimension d, eps2 = fl(ε*ε) and largest
// centred FP32 row norm R; false when FP32 cannot separate pairs at this ε.
bool filter_thresholds(uint32_t d, double eps2, double R, float* t_lo, float* t_hi);

// ---- join.cu
namespace join {
int chunk_for(bool fp64, uint32_t dpad);
void run(mistic_handle_s*, bool fp64, int CH, const JoinParams&);
// FP64 decision of the band list left by the FP32 / tensor-core joins.
void run_band(mistic_handle_s*, const JoinParams&);
// Tensor-core join over TcParams.units; KP = augmented K (d + 2 rounded up to 16).
bool tc_supported(uint32_t d);
int tc_kp(uint32_t d);
uint32_t tc_rows(uint32_t d);
void run_tc(mistic_handle_s*, const JoinParams&, const TcParams&);
// Long rows (tc_kp(d) > 128) and the tf32 mode: K-chunked kernel over rows
// prepared once at operand precision `prec` (0: bf16 hi and lo in xh, xl;
// 1: bf16 in xh; 2: tf32-rounded FP32 in xh; n x tcw_kd(d, prec) elements
// each) with their FP32 norms in xn.
uint32_t tcw_kd(uint32_t d, int prec);
void tcw_prepare(mistic_handle_s*, int prec, const float* xf, uint32_t dpad32, uint32_t d, size_t n, void* xh,
                 void* xl, float* xn);
void run_tcw(mistic_handle_s*, const JoinParams&, const TcParams&);
}  // namespace join

// ---- brute.cu: FP64 brute-force neighbour counts of rows [row0, row1)
// against all n rows (device input, device counts).
void bruteforce_rows(mistic_handle_s* h, const void* x, mistic_dtype dt, uint64_t n, uint32_t d, double eps2,
                     uint64_t row0, uint64_t row1, uint32_t* counts);

// ---- rp.cpp: reference-point selection on the host.
// stats: per-dim mean (d), min (d), max (d); cov: d x d sample covariance.
// The reference's per-layer candidate scoring on a host copy of the data
// sample (S x d rows): k points chosen greedily (MISTIC_RP_SCORED).
void select_reference_points_scored(const mistic_opts& o, uint32_t d, uint32_t k, double eps,
                                    const std::vector<double>& mean, const std::vector<double>& mn,
                                    const std::vector<double>& mx, const std::vector<double>& cov,
                                    const std::vector<double>& sample, uint32_t S, std::vector<double>& rps);
void select_reference_points(const mistic_opts& o, uint32_t d, uint32_t k,
                             const std::vector<double>& mean,
                             const std::vector<double>& mn,
                             const std::vector<double>& mx,
                             const std::vector<double>& cov,
                             std::vector<double>& rps);

}  // namespace mistic
