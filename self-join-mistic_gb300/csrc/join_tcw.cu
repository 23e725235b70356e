// Tensor-core distance join for long rows (d + 2 > 128): K-chunked Gram tiles.
//
// Reference counterpart: the FP64 distance loop of nodeByPoint5 /
// cachedDistanceCheck (src/kernel.cu:992-1046, 833-865).  For long rows a
// unit -- up to 256 points of one large home bin against a segment of its
// neighbour bins (bins >= home) -- is a dense contraction:
//
//   G[m][n] = a_m . q_n   (K = d, rows relative to the bounding-box centre)
//   D'[m][n] = |a_m|^2 - 2 G[m][n] + (|q_n|^2 - T(n))
//
// and a pair is a candidate when D' < 0.  The sorted FP32 rows are split
// once into bf16 hi and lo arrays (k_split_rows) with their FP32 norms;
// G = Ahi.Bhi + Ahi.Blo + Alo.Bhi is accumulated in FP32 in tensor memory.
// Unlike the short-row kernel (join_tc.cu) nothing is converted inside the
// join: operands stream from L2 into shared memory in K chunks of 32.  The
// home rows (contiguous) come as 128-row TMA tiles (cp.async.bulk.tensor,
// 64-byte rows, 64B swizzle); so do a group's candidate rows when they are
// one contiguous run of sorted rows (inside a large bin, or across bins that
// follow one another).  Candidates from scattered bins come by cp.async in
// 16-byte chunks written to the same swizzled layout (the MMAs ran 25% faster
// on it than on no-swizzle core matrices).  TMA 4-row gathers of scattered
// candidate rows were measured slower: 64-byte rows keep the copy engine busy
// far longer than the MMAs take.
//
// Tiles: 2 home chunks of 128 rows (MMA M = 128 each) x up to 256 candidate
// columns (MMA N), i.e. two 128 x 256 FP32 accumulators = all 512 TMEM
// columns.  A stage holds one K chunk of both home chunks and of the 256
// candidate rows (64 KB); three stages are in flight.
//
// Operand precision (template PREC, chosen per call by the host):
//   0  split bf16: G = Ahi.Bhi + Ahi.Blo + Alo.Bhi, 3 MMAs per K step of 16,
//      stages of K = 32 as 64-byte rows (64B swizzle); operand error
//      3.02 * 2^-16 of |a_k||q_k| (bf16 keeps 8 significant bits: the hi part
//      is within 2^-8, hi + lo within 2^-16 of the value);
//   1  single bf16: one MMA per K step of 16, stages of K = 64 as 128-byte
//      rows (128B swizzle); a third of the tensor work, operand error
//      2^-7 + 2^-16 -- used when the resulting band stays narrow (large eps
//      relative to the rows' norms);
//   2  tf32 (kind::tf32, rows rounded to tf32 once): one MMA per K step of 8,
//      stages of K = 32 as 128-byte rows; operand error 2^-10 + 2^-22.
// All three stage 64 KB a stage (home tiles 32 KB, candidates 32 KB).
//
// Exactness: the same rigorous bound as the short-row kernel (the operand
// error above, 2^-19 per MMA instruction of accumulation, FP32 norms, global
// FP32 centring), plus the FP32 epilogue arithmetic (accounted for in
// TcParams.kappa by the host): D' <= -dlt(n) accepts, D' < 0 otherwise goes
// to the band list, whose pairs are re-decided with the reference FP64
// predicate.  Columns whose bound exceeds 0.1 eps2 are re-decided entirely
// in FP64.
#include <cuda.h>
#include <cudaTypedefs.h>
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <mutex>
#include <cstdio>
#include <cstdlib>

#include "emit.cuh"
#include "internal.cuh"
#include "tc_common.cuh"

namespace mistic {
namespace {

using namespace tcu;

constexpr int WM = 128;      // rows per home chunk (MMA M)
constexpr int WG = 2;        // home chunks per unit
constexpr int WN = 256;      // candidate columns per group (MMA N at most)
constexpr int WKC = 32;      // K per pipeline stage of the split kernel (two MMA K steps of 16)
constexpr int WNS = 3;       // stages
constexpr int WWIN = 256;    // neighbour bins per candidate window
constexpr int WNPW = 8;      // producer warps: thread t loads home row t and candidate row t
constexpr int WNPROD = WNPW * 32;
constexpr int WNEPI = 16;    // epilogue warps: 4 TMEM lane quarters x 4 column groups
constexpr int WEPI0 = WNPW;  // first epilogue warp (a multiple of 4: warp % 4 is its lane quarter)
constexpr int WMMA = WEPI0 + WNEPI;
constexpr int WTHREADS = (WMMA + 1) * 32;
constexpr int WGS = 2;       // group metadata slots
// stage layout (bytes): home hi | home lo (by TMA) | candidates hi |
// candidates lo (by cp.async), all as 64-byte rows in the 64B swizzle
constexpr uint32_t A_CHUNK = WM * WKC * 2;      // one 128-row home chunk, hi or lo (8 KB)
constexpr uint32_t A_LO = WG * A_CHUNK;         // 16 KB
constexpr uint32_t B_HI = 2 * WG * A_CHUNK;     // 32 KB
constexpr uint32_t B_LO = B_HI + WN * WKC * 2;  // 48 KB
constexpr uint32_t STAGE_BYTES = B_LO + WN * WKC * 2;
constexpr uint32_t SW_ATOM = 8 * WKC * 2;       // 8 rows x 64 B: the home rows' swizzle atom and MMA SBO
// single-operand precisions (PREC 1, 2): 128-byte rows, home chunks 16 KB
// each at 0, 16 KB, candidates at 32 KB
constexpr uint32_t S_ACHUNK = WM * 128;         // 16 KB
constexpr uint32_t S_B = WG * S_ACHUNK;         // 32 KB
constexpr uint32_t SW_ATOM128 = 8 * 128;        // 8 rows x 128 B
constexpr uint32_t WFLAG_END = 1;
static_assert(WNPROD == WG * WM && WNPROD == WN, "one producer thread per operand row");
static_assert(S_B + WN * 128 == STAGE_BYTES, "all precisions stage the same bytes");

// K elements per stage, by precision
__host__ __device__ constexpr uint32_t tcw_kstage(int prec) { return prec == 1 ? 64u : 32u; }

// Everything the epilogue needs about one group (a unit's home rows x up to
// 256 candidate columns).  Written by the producers before the group's first
// stage is published; released by the epilogue (gfree) when it is done.
struct __align__(16) WGroup {
  uint32_t qid[WN];      // original ids of the candidates
  float hq[WN];          // |q|^2 - T(n)
  float dlt[WN];         // accept when D' <= -dlt
  uint32_t aid[WG * WM]; // original ids of the home rows
  float na[WG * WM];     // |a|^2 of the home rows
  uint32_t a0, nrows, ncols, ng, flags;
  uint32_t hlo, hhi, hq0;  // columns [hlo, hhi) are home-bin rows, column hlo at sorted position hq0
  uint32_t tag;            // the pair ring's tag of the group's unit (0 outside ring mode)
};

struct WShared {
  WGroup grp[WGS];
  uint32_t w_start[WWIN];
  uint32_t w_pref[WWIN + 1];
  uint32_t scan_ws[WNPW];
  unsigned long long unit;
  uint32_t w_home;   // (window generation << 8) | index of the home bin in the window
  uint32_t ra2max;   // float bits, non-negative
  uint32_t abort_flag;
  uint32_t tmem_base;
  uint32_t pflag[2];
  unsigned long long full[WNS], afull[WNS], sfree[WNS], dfull[WG], dfree[WG], gfree[WGS], gready[WGS];
};

__device__ __forceinline__ void wprod_sync() { asm volatile("bar.sync 1, %0;" ::"n"(WNPROD) : "memory"); }

// wprod_sync that also returns the AND of p over all producer threads
__device__ __forceinline__ bool wprod_sync_and(bool p) {
  uint32_t r;
  asm volatile(
      "{\n\t.reg .pred pi, po;\n\t"
      "setp.ne.u32 pi, %1, 0;\n\t"
      "bar.red.and.pred po, 1, %2, pi;\n\t"
      "selp.u32 %0, 1, 0, po;\n\t}"
      : "=r"(r)
      : "r"((uint32_t)p), "n"(WNPROD)
      : "memory");
  return r != 0u;
}

// The tensor maps over the split rows (hi, lo): home-row tiles of 128 rows x
// 32 bf16, 64B swizzle.
struct TcwMaps {
  CUtensorMap ah, al;
};

// tcgen05 shared-memory descriptor, K-major, 64B swizzle: 64-byte rows,
// 8-row atoms of 512 B (SBO); LBO is not used by swizzled K-major layouts.
__device__ __forceinline__ uint64_t desc_sw64(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((SW_ATOM >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version
  d |= (uint64_t)4 << 61;  // layout: 64B swizzle
  return d;
}

// The same for 128-byte rows, 128B swizzle: 8-row atoms of 1024 B (SBO).
__device__ __forceinline__ uint64_t desc_sw128(uint32_t saddr) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)1 << 16;
  d |= (uint64_t)((SW_ATOM128 >> 4) & 0x3FFF) << 32;
  d |= (uint64_t)1 << 46;  // descriptor version
  d |= (uint64_t)2 << 61;  // layout: 128B swizzle
  return d;
}

__device__ __forceinline__ void cp_async16_s(uint32_t dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}

// Arrive on `bar` once every cp.async this thread issued before has
// completed (the barrier's expected count is not raised: the arrival counts
// as one of its initial ones).
__device__ __forceinline__ void cp_async_arrive_noinc(unsigned long long* bar) {
  asm volatile("cp.async.mbarrier.arrive.noinc.shared::cta.b64 [%0];" ::"r"(smem_u32(bar)) : "memory");
}

__device__ __forceinline__ void mbar_expect_tx(uint32_t mbar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;" ::"r"(mbar), "r"(bytes) : "memory");
}

// 2-D tile load (x: first element, a multiple of 8 bf16; y: first row).
__device__ __forceinline__ void tma_tile_2d(uint32_t dst, uint64_t map, int x, int y, uint32_t mbar) {
  asm volatile(
      "cp.async.bulk.tensor.2d.shared::cluster.global.tile.mbarrier::complete_tx::bytes [%0], [%1, {%2, %3}], [%4];" ::"r"(
          dst),
      "l"(map), "r"(x), "r"(y), "r"(mbar)
      : "memory");
}

// One warp per sorted row: bf16 hi/lo split of the FP32 row (zero beyond its
// dpad32 stored values, up to kd) into the row-major arrays xh, xl (kd bf16
// a row; xl null: the hi part alone, for the single-bf16 precision), and its
// FP32 squared norm.
__global__ void k_split_rows(const float* __restrict__ xf, uint32_t dpad32, uint32_t kd, size_t n,
                             uint4* __restrict__ xh, uint4* __restrict__ xl, float* __restrict__ xn) {
  const size_t row = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* x = xf + row * dpad32;
  uint4* oh_row = xh + row * (kd / 8);
  uint4* ol_row = xl + row * (kd / 8);
  float acc = 0.f;
  for (uint32_t kb = lane; kb < kd / 8; kb += 32) {
    float v[8];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t k0 = kb * 8 + 4 * h;
      float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
      if (k0 < dpad32) f = *reinterpret_cast<const float4*>(x + k0);  // dpad32 % 4 == 0, zero beyond d
      v[4 * h] = f.x, v[4 * h + 1] = f.y, v[4 * h + 2] = f.z, v[4 * h + 3] = f.w;
    }
    uint4 oh, ol;
    uint32_t* ph = reinterpret_cast<uint32_t*>(&oh);
    uint32_t* pl = reinterpret_cast<uint32_t*>(&ol);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      acc = fmaf(v[2 * i], v[2 * i], acc);
      acc = fmaf(v[2 * i + 1], v[2 * i + 1], acc);
      const __nv_bfloat162 hv = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
      const float2 hf = __bfloat1622float2(hv);
      const __nv_bfloat162 lv = __floats2bfloat162_rn(v[2 * i] - hf.x, v[2 * i + 1] - hf.y);
      ph[i] = *reinterpret_cast<const uint32_t*>(&hv);
      pl[i] = *reinterpret_cast<const uint32_t*>(&lv);
    }
    oh_row[kb] = oh;
    if (xl) ol_row[kb] = ol;
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(FULL_MASK, acc, o);
  if (lane == 0) xn[row] = acc;
}

// One warp per sorted row: the FP32 row rounded to tf32 (round to nearest,
// ties away; the low 13 bits are zero, so the tensor core reads it exactly),
// zero beyond dpad32 up to kd, and its FP32 squared norm (of the unrounded
// values).
__global__ void k_tf32_rows(const float* __restrict__ xf, uint32_t dpad32, uint32_t kd, size_t n,
                            float4* __restrict__ xt, float* __restrict__ xn) {
  const size_t row = (size_t)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5);
  const int lane = threadIdx.x & 31;
  if (row >= n) return;
  const float* x = xf + row * dpad32;
  float4* o_row = xt + row * (kd / 4);
  float acc = 0.f;
  for (uint32_t c = lane; c < kd / 4; c += 32) {
    float4 f = make_float4(0.f, 0.f, 0.f, 0.f);
    if (4 * c < dpad32) f = *reinterpret_cast<const float4*>(x + 4 * c);  // dpad32 % 4 == 0
    acc = fmaf(f.x, f.x, acc);
    acc = fmaf(f.y, f.y, acc);
    acc = fmaf(f.z, f.z, acc);
    acc = fmaf(f.w, f.w, acc);
    float v[4] = {f.x, f.y, f.z, f.w};
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      uint32_t t;
      asm("cvt.rna.tf32.f32 %0, %1;" : "=r"(t) : "f"(v[i]));
      v[i] = __uint_as_float(t);
    }
    o_row[c] = make_float4(v[0], v[1], v[2], v[3]);
  }
#pragma unroll
  for (int o = 16; o; o >>= 1) acc += __shfl_xor_sync(FULL_MASK, acc, o);
  if (lane == 0) xn[row] = acc;
}

// ---------------------------------------------------------------- pipeline
// One persistent CTA per SM: 8 producer warps, 16 epilogue warps, 1 MMA warp.
//   producers  fetch units; per group of up to 256 candidates all 8 warps
//              compute the columns' sorted positions, ids, norms and
//              thresholds; then, per K chunk, thread 0 issues the stage's
//              TMA tiles (home rows, and the candidate rows of a contiguous
//              group) against one expect_tx on afull, and every producer
//              thread copies its scattered candidate rows by cp.async;
//   MMA warp   one lane issues 2 x 3 tcgen05.mma (K 16, M 128, N up to 256)
//              per home chunk and stage, commits each stage to sfree and, at
//              a group's last stage, each accumulator to dfull;
//   epilogue   tcgen05.ld of TMEM lane quarter w % 4, D' = |a|^2 - 2G + hq,
//              sign-bit test, home-bin rule by column range, sure accepts
//              to the pair list, the error band to the band list.
// Barriers (all waits bounded by a %globaltimer deadline):
//   full[s]   producers -> MMA       (WNPROD cp.async arrivals: candidate rows landed)
//   afull[s]  producer 0 -> MMA      (one arrive.expect_tx + the bytes of the stage's TMA tiles)
//   gready[x] producers -> MMA       (WNPROD arrivals: group slot x written)
//   sfree[s]  MMA -> producers       (tcgen05.commit: stage s read)
//   dfull[g]  MMA -> epilogue        (tcgen05.commit, or a plain arrive to stop)
//   dfree[g]  epilogue -> MMA        (WNEPI arrivals; accumulator g reusable)
//   gfree[x]  epilogue -> producers  (WNEPI arrivals; group slot x reusable)
template <int PREC>
__global__ void __launch_bounds__(WTHREADS, 1)
    k_join_tcw(const JoinParams P, const TcParams T, const __grid_constant__ TcwMaps M) {
  constexpr uint32_t KST = tcw_kstage(PREC);     // K elements per stage
  constexpr uint32_t ESZ = PREC == 2 ? 4u : 2u;  // operand element bytes
  extern __shared__ __align__(1024) unsigned char tcw_dyn[];
  __shared__ WShared S;
  // stages: WNS x STAGE_BYTES from the first 1024-byte boundary (swizzle atoms
  // must sit on their natural alignment); then the pair staging buffers
  const uint32_t dyn0 = smem_u32(tcw_dyn);
  const uint32_t stage_base = (dyn0 + 1023u) & ~1023u;
  unsigned long long* pstage = reinterpret_cast<unsigned long long*>(tcw_dyn + (stage_base - dyn0) + WNS * STAGE_BYTES);
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const uint32_t nkc = T.kd / KST;   // stages per group
  volatile uint32_t* abort_flag = &S.abort_flag;

  if (tid == 0) {
    for (int i = 0; i < WNS; ++i) {
      mbar_init(&S.full[i], WNPROD);
      mbar_init(&S.afull[i], 1);
      mbar_init(&S.sfree[i], 1);
    }
    for (int i = 0; i < WG; ++i) {
      mbar_init(&S.dfull[i], 1);
      mbar_init(&S.dfree[i], WNEPI);
    }
    for (int i = 0; i < WGS; ++i) {
      mbar_init(&S.gfree[i], WNEPI);
      mbar_init(&S.gready[i], WNPROD);
    }
    asm volatile("fence.mbarrier_init.release.cluster;");
    S.abort_flag = 0;
    S.w_home = 0xffffffffu;
  }
  if (warp == WMMA) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&S.tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = S.tmem_base;

  if (warp < WNPW) {
    // ============================ producers
    // All 8 warps prepare each group (candidate positions, ids, thresholds);
    // warp 0 then issues the group's stages as TMA copies.  Every branch that
    // leads to bar.sync is taken on a value all producer threads hold in
    // registers or read from shared memory after the same bar.sync; barrier
    // waits shared by all producers are done by thread 0 and broadcast
    // through S.pflag[2] (a thread is at most one bar.sync behind thread 0).
    const uint32_t t = (uint32_t)tid;
    uint32_t step = 0, group = 0, pf = 0, wgen = 0;
    unsigned long long n_tiles = 0, n_cells = 0;
    bool aborted = false;
    long long pc_grp = 0, pc_sfree = 0, pc_issue = 0, pc_pub = 0;  // cycles (T.prof)
    const long long p_start = T.prof ? clock64() : 0;
    const uint64_t map_ah = reinterpret_cast<uint64_t>(&M.ah), map_al = reinterpret_cast<uint64_t>(&M.al);
    // thread 0 waits on b (bounded), all producers learn the outcome; once
    // the CTA aborts every such wait fails (thread 0 may have given up alone
    // while issuing a contiguous group's stages)
    auto shared_wait = [&](unsigned long long* b, uint32_t parity) -> bool {
      const uint32_t sl = pf++ & 1;
      if (tid == 0) S.pflag[sl] = (!*abort_flag && wait_or_abort(b, parity, abort_flag, T.wait_limit)) ? 1u : 0u;
      wprod_sync();
      return S.pflag[sl] != 0u;
    };
    // the same, also returning the AND of p over the producers
    auto shared_wait_and = [&](unsigned long long* b, uint32_t parity, bool p, bool* all) -> bool {
      const uint32_t sl = pf++ & 1;
      if (tid == 0) S.pflag[sl] = (!*abort_flag && wait_or_abort(b, parity, abort_flag, T.wait_limit)) ? 1u : 0u;
      *all = wprod_sync_and(p);
      return S.pflag[sl] != 0u;
    };
    const uint16_t* XH = static_cast<const uint16_t*>(T.xh);
    const uint16_t* XL = static_cast<const uint16_t*>(T.xl);
    const unsigned char* XS = static_cast<const unsigned char*>(T.xh);  // single-operand rows (bf16 or tf32)
    // split: lane l moves rows 32 w + l / 4 + 8 i (i < 4), piece l % 4;
    // single: rows 32 w + l / 8 + 4 i (i < 8), 16-byte chunk l % 8
    const uint32_t prow0 = 32u * (uint32_t)warp + ((uint32_t)lane >> (PREC == 0 ? 2 : 3));
    const uint32_t pkb = ((uint32_t)lane >> 1) & 1u, ph = (uint32_t)lane & 1u;
    const uint32_t pch = (uint32_t)lane & 7u;
    for (;;) {
      const uint32_t slot = pf++ & 1;
      if (tid == 0) {
        // claim index -> unit: units deferred by the last ring pass first,
        // then the list from main_start (the identity outside ring mode)
        const unsigned long long t = atomicAdd(&T.ctr->next_unit, 1ull);
        const unsigned long long uu = t < T.n_def_in ? (unsigned long long)T.def_in[t] : T.main_start + (t - T.n_def_in);
        S.unit = uu;
        S.ra2max = 0;
        bool go = (T.claim_cap == 0 || t < T.claim_cap) && uu < T.n_units && !*abort_flag;
        if (go && P.ring && *(volatile unsigned long long*)&P.ctr->stop) {  // the ring filled: leave it for the next pass
          const RingCtx rc{P.pair_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
          ring_defer(&rc, P.tag_base_tc + (uint32_t)uu);
          go = false;
        }
        S.pflag[slot] = go ? 1u : 0u;
      }
      wprod_sync();
      if (!S.pflag[slot]) break;
      const Unit U = T.units[S.unit];
      const uint32_t hs = P.bstart[U.h], he = P.bstart[U.h + 1];
      const uint32_t a0 = hs + U.chunk * (WG * WM);
      const uint32_t nrows = min((uint32_t)(WG * WM), he - a0);
      const uint32_t ng = (nrows + WM - 1) / WM;
      const bool arow = t < nrows;
      const uint32_t my_aid = arow ? P.ids[a0 + t] : 0u;
      const float my_na = arow ? T.xn[a0 + t] : 0.f;
      {
        float m = my_na;
#pragma unroll
        for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL_MASK, m, o));
        if (lane == 0) atomicMax(&S.ra2max, __float_as_uint(m));
      }
      wprod_sync();
      const float ra2max = __uint_as_float(S.ra2max);

      uint32_t seg_next = U.s0, w_nb = 0, w_pos = 0, w_total = 0;
      int w_hj = -1;
      while (w_pos < w_total || seg_next < U.s1) {
        if (w_pos >= w_total) {  // next window of up to WWIN neighbour bins
          const uint32_t nb = min((uint32_t)WWIN, U.s1 - seg_next);
          uint32_t st0 = 0, sz0 = 0, bn = 0xffffffffu;
          if (t < nb) {
            bn = P.nbr[seg_next + t];
            st0 = P.bstart[bn];
            sz0 = P.bstart[bn + 1] - st0;
          }
          const uint32_t incl = warp_scan_incl(sz0);
          if (lane == 31) S.scan_ws[warp] = incl;
          wprod_sync();
          uint32_t wp = 0;
          for (int w = 0; w < warp; ++w) wp += S.scan_ws[w];
          ++wgen;
          if (t < nb) {
            S.w_start[t] = st0;
            S.w_pref[t + 1] = wp + incl;
            if (bn == U.h) S.w_home = ((wgen & 0xffffffu) << 8) | t;
          }
          if (tid == 0) S.w_pref[0] = 0;
          wprod_sync();
          {
            const uint32_t wh = S.w_home;
            w_hj = (wh >> 8) == (wgen & 0xffffffu) ? (int)(wh & 255u) : -1;
          }
          w_nb = nb;
          w_pos = 0;
          w_total = S.w_pref[nb];
          seg_next += nb;
        }
        // ---- a group: columns [w_pos, w_pos + ncols) of the window
        const long long cg0 = T.prof ? clock64() : 0;
        const uint32_t ncols = min((uint32_t)WN, w_total - w_pos);
        const bool bcol = t < ncols;
        // sorted position of column t (columns past ncols: the first one,
        // never loaded)
        uint32_t q = 0;
        {
          const uint32_t rank = w_pos + (bcol ? t : 0u);
          int lo = 0, hi = (int)w_nb - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S.w_pref[mid] <= rank) lo = mid; else hi = mid - 1;
          }
          q = S.w_start[lo] + (rank - S.w_pref[lo]);
        }
        // the group's candidates are one contiguous run of sorted rows (the
        // common case inside large bins) when every column sits at the first
        // one's position + its index: then the stages fetch them as 128-row
        // TMA tiles like the home rows
        uint32_t qf;
        {
          int lo = 0, hi = (int)w_nb - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S.w_pref[mid] <= w_pos) lo = mid; else hi = mid - 1;
          }
          qf = S.w_start[lo] + (w_pos - S.w_pref[lo]);
        }
        const bool in_run = !bcol || q == qf + t;
        float hqv = 0.f, dl = 0.f;
        uint32_t qid = 0;
        if (bcol) {
          qid = P.ids[q];
          const float nq2 = T.xn[q];
          float tcol;
          if (column_threshold(T.b, ra2max, nq2, &tcol, &dl)) {
            hqv = nq2 - tcol;
          } else {
            hqv = -1e30f;   // every row of this column becomes a candidate ...
            dl = INFINITY;  // ... and none is accepted without the FP64 check
          }
        }
        const uint32_t gs = group % WGS;
        bool b_tma = false;
        if (!shared_wait_and(&S.gfree[gs], ((group / WGS) & 1) ^ 1, in_run, &b_tma)) {
          aborted = true;
          break;
        }
        WGroup& Gm = S.grp[gs];
        Gm.qid[t] = qid;
        Gm.hq[t] = hqv;
        Gm.dlt[t] = dl;
        Gm.aid[t] = my_aid;
        Gm.na[t] = my_na;
        if (tid == 0) {
          uint32_t hlo = 0, hhi = 0, hq0 = 0;
          if (w_hj >= 0) {
            const uint32_t hr0 = S.w_pref[w_hj], hr1 = S.w_pref[w_hj + 1];
            const uint32_t lo = max(hr0, w_pos), hi = min(hr1, w_pos + ncols);
            if (lo < hi) {
              hlo = lo - w_pos;
              hhi = hi - w_pos;
              hq0 = hs + (lo - hr0);
            }
          }
          Gm.a0 = a0;
          Gm.nrows = nrows;
          Gm.ncols = ncols;
          Gm.ng = ng;
          Gm.flags = 0;
          Gm.hlo = hlo;
          Gm.hhi = hhi;
          Gm.hq0 = hq0;
          Gm.tag = P.ring ? P.tag_base_tc + (uint32_t)S.unit : 0u;
          n_tiles += (unsigned long long)ng * ((ncols + 127) / 128);
          n_cells += (unsigned long long)nrows * ncols;
        }
        mbar_arrive(&S.gready[gs]);  // releases this thread's writes of the group slot
        if (T.prof) pc_grp += clock64() - cg0;
        // ---- the group's K chunks, one stage each: the home rows as 128-row
        // TMA tiles (thread 0, against one expect_tx on afull), the candidate
        // rows by cp.async, lane l of warp w moving rows 32w + 8i + l / 4
        // (i = 0..3), piece l % 4 (K block 2j + (l % 4) / 2 of pair j, hi or
        // lo by l % 2): 8 rows x 32 bytes of hi and of lo per instruction
        constexpr int NBR = PREC == 0 ? 4 : 8;  // candidate rows this thread moves
        constexpr uint32_t RSTEP = PREC == 0 ? 8u : 4u;
        const unsigned char* b_src[NBR];
        uint32_t b_ok = 0;
#pragma unroll
        for (int i = 0; i < NBR; ++i) {
          // column prow0 + RSTEP i is owned by lane RSTEP i + lane / (32 / RSTEP) of this warp
          const uint32_t qi = __shfl_sync(FULL_MASK, q, (int)(RSTEP * i) + (lane >> (PREC == 0 ? 2 : 3)));
          if (PREC == 0)
            b_src[i] = reinterpret_cast<const unsigned char*>((ph ? XL : XH) + (size_t)qi * T.kd);
          else
            b_src[i] = XS + ((size_t)qi * T.kd + 0) * ESZ + 16u * pch;
          if (prow0 + RSTEP * i < ncols) b_ok |= 1u << i;
        }
        const uint32_t nbt = b_tma ? (ncols + WM - 1) / WM : 0u;  // candidate tiles by TMA
        const uint32_t abytes = (ng + nbt) * 2u * A_CHUNK;  // 16 KB a 128-row tile at every precision
        if (b_tma) {
          // every copy of the group's stages is a TMA tile: thread 0 alone
          // waits for each stage, issues its tiles and makes all WNPROD
          // arrivals on its full barrier; the other producers go on to the
          // next group (whose slot barrier thread 0 joins when done).  A
          // failed wait leaves the CTA's abort flag set, which fails the next
          // shared wait of every producer.
          if (tid == 0) {
            for (uint32_t kc = 0; kc < nkc; ++kc) {
              const uint32_t s = step % WNS;
              const long long cs0 = T.prof ? clock64() : 0;
              if (!wait_or_abort(&S.sfree[s], ((step / WNS) & 1) ^ 1, abort_flag, T.wait_limit)) break;
              const long long cs1 = T.prof ? clock64() : 0;
              const uint32_t sb = stage_base + s * STAGE_BYTES;
              const uint32_t ab = smem_u32(&S.afull[s]);
              mbar_expect_tx(ab, abytes);
              for (uint32_t g = 0; g < ng; ++g) {
                if (PREC == 0) {
                  tma_tile_2d(sb + g * A_CHUNK, map_ah, (int)(kc * WKC), (int)(a0 + g * WM), ab);
                  tma_tile_2d(sb + A_LO + g * A_CHUNK, map_al, (int)(kc * WKC), (int)(a0 + g * WM), ab);
                } else {
                  tma_tile_2d(sb + g * S_ACHUNK, map_ah, (int)(kc * KST), (int)(a0 + g * WM), ab);
                }
              }
              // the candidate rows [qf, qf + 128 nbt): rows past ncols are
              // fetched (or zero-filled past the last row) and never read
              for (uint32_t b = 0; b < nbt; ++b) {
                const int y = (int)(qf + b * WM);
                if (PREC == 0) {
                  tma_tile_2d(sb + B_HI + b * A_CHUNK, map_ah, (int)(kc * WKC), y, ab);
                  tma_tile_2d(sb + B_LO + b * A_CHUNK, map_al, (int)(kc * WKC), y, ab);
                } else {
                  tma_tile_2d(sb + S_B + b * S_ACHUNK, map_ah, (int)(kc * KST), y, ab);
                }
              }
              mbar_arrive_n(&S.full[s], WNPROD);
              ++step;
              if (T.prof) {
                const long long cs2 = clock64();
                pc_sfree += cs1 - cs0;
                pc_issue += cs2 - cs1;
              }
            }
          } else {
            step += nkc;
          }
          w_pos += ncols;
          ++group;
          continue;
        }
        for (uint32_t kc = 0; kc < nkc; ++kc) {
          const uint32_t s = step % WNS;
          const long long cs0 = T.prof ? clock64() : 0;
          if (!shared_wait(&S.sfree[s], ((step / WNS) & 1) ^ 1)) {
            aborted = true;
            break;
          }
          const long long cs1 = T.prof ? clock64() : 0;
          const uint32_t sb = stage_base + s * STAGE_BYTES;
          if (tid == 0) {
            const uint32_t ab = smem_u32(&S.afull[s]);
            mbar_expect_tx(ab, abytes);
            for (uint32_t g = 0; g < ng; ++g) {
              if (PREC == 0) {
                tma_tile_2d(sb + g * A_CHUNK, map_ah, (int)(kc * WKC), (int)(a0 + g * WM), ab);
                tma_tile_2d(sb + A_LO + g * A_CHUNK, map_al, (int)(kc * WKC), (int)(a0 + g * WM), ab);
              } else {
                tma_tile_2d(sb + g * S_ACHUNK, map_ah, (int)(kc * KST), (int)(a0 + g * WM), ab);
              }
            }
          }
          if (PREC == 0) {
            const uint32_t bdst = sb + (ph ? B_LO : B_HI);
#pragma unroll
            for (int j = 0; j < WKC / 16; ++j) {
              const uint32_t kb = 2 * j + pkb;  // K block within the stage
#pragma unroll
              for (int i = 0; i < NBR; ++i) {
                const uint32_t r = prow0 + 8 * i;  // 64-byte row r, 16-byte chunk kb, 64B swizzle
                const uint32_t off = r * 64u + ((kb ^ ((r >> 1) & 3u)) << 4);
                if (b_ok & (1u << i))
                  cp_async16_s(bdst + off, b_src[i] + (size_t)(kc * WKC + kb * 8) * 2);
              }
            }
          } else {
            // 128-byte rows: 16-byte chunk pch of row r at r * 128 + 16 (pch ^ (r & 7))
#pragma unroll
            for (int i = 0; i < NBR; ++i) {
              const uint32_t r = prow0 + RSTEP * i;
              const uint32_t off = r * 128u + ((pch ^ (r & 7u)) << 4);
              if (b_ok & (1u << i)) cp_async16_s(sb + S_B + off, b_src[i] + (size_t)kc * KST * ESZ);
            }
          }
          // this thread's arrival on the stage's full barrier is made by the
          // copy engine once its copies above have landed: producers never
          // block on their own copies, so all WNS stages can be in flight
          cp_async_arrive_noinc(&S.full[s]);
          ++step;
          const long long cs2 = T.prof ? clock64() : 0;
          if (T.prof) {
            pc_sfree += cs1 - cs0;
            pc_issue += cs2 - cs1;
            pc_pub += clock64() - cs2;
          }
        }
        if (aborted) break;
        w_pos += ncols;
        ++group;
      }
      if (aborted) break;
    }
    if (!aborted) {
      // stop marker: a group slot flagged END behind a stage with no copies
      const uint32_t gs = group % WGS, s = step % WNS;
      bool ok = shared_wait(&S.gfree[gs], ((group / WGS) & 1) ^ 1);
      if (ok) ok = shared_wait(&S.sfree[s], ((step / WNS) & 1) ^ 1);
      if (ok) {
        if (tid == 0) S.grp[gs].flags = WFLAG_END;
        mbar_arrive(&S.gready[gs]);
        mbar_arrive(&S.full[s]);
        if (tid == 0) mbar_arrive(&S.afull[s]);
      }
    }
    asm volatile("cp.async.wait_all;" ::: "memory");
    // an aborting CTA may still have TMA copies in flight into its stages:
    // wait (bounded) until each stage's last issued home tiles have landed
    if (tid == 0 && *abort_flag) {
      volatile uint32_t no_abort = 0;
      for (uint32_t j = step > WNS ? step - WNS : 0; j < step; ++j)
        wait_or_abort(&S.afull[j % WNS], (j / WNS) & 1, &no_abort, T.wait_limit);
    }
    if (tid == 0 && n_tiles) {
      atomicAdd(&T.ctr->tiles, n_tiles);
      atomicAdd(&T.ctr->cells, n_cells);
    }
    if (tid == 0 && T.prof) {
      atomicAdd(&T.ctr->prof[1], (unsigned long long)(clock64() - p_start));
      atomicAdd(&T.ctr->prof[7], (unsigned long long)pc_grp);
      atomicAdd(&T.ctr->prof[0], (unsigned long long)pc_sfree);
      atomicAdd(&T.ctr->prof[9], (unsigned long long)pc_issue);
      atomicAdd(&T.ctr->prof[14], (unsigned long long)pc_pub);
    }
  } else if (warp == WMMA) {
    // ============================ MMA issuer
    if (lane == 0) {
      uint32_t step = 0, group = 0;
      uint32_t use[WG] = {0, 0};
      unsigned long long* last_bar = nullptr;
      uint32_t last_par = 0;
      // failure-detection test: the lane signals nothing, so the producers'
      // and the epilogue's bounded waits run out
      bool ok = !T.stall_test;
      long long mw_full = 0, mw_dfree = 0;
      const long long m_start = T.prof ? clock64() : 0;
      while (ok) {
        uint32_t s = step % WNS;
        const long long c0 = T.prof ? clock64() : 0;
        ok = wait_or_abort(&S.full[s], (step / WNS) & 1, abort_flag, T.wait_limit) &&
             wait_or_abort(&S.afull[s], (step / WNS) & 1, abort_flag, T.wait_limit);
        if (T.prof) mw_full += clock64() - c0;
        // the group slot's metadata (written before the group's first stage)
        if (ok) ok = wait_or_abort(&S.gready[group % WGS], (group / WGS) & 1, abort_flag, T.wait_limit);
        if (!ok) break;
        const WGroup& Gm = S.grp[group % WGS];
        if (Gm.flags & WFLAG_END) {
          // wake the epilogue on accumulator 0 only once every epilogue warp
          // has taken its previous use: an earlier arrival would complete a
          // second phase of dfull[0] under a warp still waiting for the
          // first (parity aliasing)
          wait_or_abort(&S.dfree[0], (use[0] & 1) ^ 1, abort_flag, T.wait_limit);
          mbar_arrive(&S.dfull[0]);
          break;
        }
        const uint32_t ng = Gm.ng;
        const uint32_t nmma = max(16u, (Gm.ncols + 15u) & ~15u);  // MMA N: the group's columns, rounded to 16
        const uint32_t idesc = umma_idesc_fmt(WM, (int)nmma, PREC == 2 ? 2u : 1u);
        // MMAs of home chunk g for K chunk kc from stage s
        auto issue = [&](uint32_t g, uint32_t kc, uint32_t s) {
          const uint32_t sb = stage_base + s * STAGE_BYTES;
          const uint32_t bh = sb + B_HI, bl = sb + B_LO;
          const uint32_t dt = tbase + g * WN;
          if (PREC == 0) {
            const uint32_t ah = sb + g * A_CHUNK, al = sb + A_LO + g * A_CHUNK;
#pragma unroll
            for (int ks = 0; ks < WKC / 16; ++ks) {
              // K step of 16 bf16: 32 bytes into the 64-byte swizzled rows of
              // both operands
              const uint32_t ok16 = ks * 32;
              const uint64_t dah = desc_sw64(ah + ok16), dal = desc_sw64(al + ok16);
              const uint64_t dbh = desc_sw64(bh + ok16), dbl = desc_sw64(bl + ok16);
              mma_bf16(dt, dah, dbh, idesc, (kc | ks) ? 1u : 0u);
              mma_bf16(dt, dah, dbl, idesc, 1u);
              mma_bf16(dt, dal, dbh, idesc, 1u);
            }
          } else {
            const uint32_t a1 = sb + g * S_ACHUNK, b1 = sb + S_B;
#pragma unroll
            for (int ks = 0; ks < 4; ++ks) {
              // one K step (16 bf16 or 8 tf32) = 32 bytes into the 128-byte
              // swizzled rows of both operands
              const uint64_t da = desc_sw128(a1 + ks * 32), db = desc_sw128(b1 + ks * 32);
              if (PREC == 2)
                mma_tf32(dt, da, db, idesc, (kc | ks) ? 1u : 0u);
              else
                mma_bf16(dt, da, db, idesc, (kc | ks) ? 1u : 0u);
            }
          }
        };
        auto release = [&](uint32_t st) {  // the stage of global step st may be refilled once its MMAs have read it
          tc_commit(&S.sfree[st % WNS]);
          last_bar = &S.sfree[st % WNS];
          last_par = (st / WNS) & 1;
        };
        // Accumulator 1 may still be drained by the epilogue when the group
        // starts; rather than wait, chunk 0 runs ahead through the stages
        // already full, and chunk 1 catches up on them (their release is
        // held back) once accumulator 1 is free.  nd stages are deferred,
        // from global step d0; all stages deferred means the ring is full,
        // and then the lane waits.
        const uint32_t step0 = step;
        uint32_t nd = 0, d0 = 0;
        auto catch_up = [&]() {
          asm volatile("tcgen05.fence::after_thread_sync;");
          for (uint32_t i = 0; i < nd; ++i) {
            issue(1, d0 + i - step0, (d0 + i) % WNS);
            release(d0 + i);
          }
          nd = 0;
        };
        for (uint32_t kc = 0; kc < nkc && ok; ++kc) {
          if (kc > 0) {
            s = step % WNS;
            const long long c1 = T.prof ? clock64() : 0;
            ok = wait_or_abort(&S.full[s], (step / WNS) & 1, abort_flag, T.wait_limit) &&
                 wait_or_abort(&S.afull[s], (step / WNS) & 1, abort_flag, T.wait_limit);
            if (T.prof) mw_full += clock64() - c1;
            if (!ok) break;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          // the candidate rows were written by cp.async (generic proxy) and
          // are read by the MMAs (async proxy): this thread has acquired them
          // through the full barrier; order them before its MMAs
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          if (kc == 0) {  // first writes of this group into accumulator 0
            const long long c2 = T.prof ? clock64() : 0;
            ok = wait_or_abort(&S.dfree[0], (use[0] & 1) ^ 1, abort_flag, T.wait_limit);
            if (T.prof) mw_dfree += clock64() - c2;
            if (!ok) break;
            asm volatile("tcgen05.fence::after_thread_sync;");
          }
          issue(0, kc, s);
          if (ng > 1) {
            if (nd > 0 && mbar_ready(&S.dfree[1], (use[1] & 1) ^ 1)) catch_up();
            if (nd > 0) {
              ++nd;  // this stage's chunk 1 waits too
            } else if (kc == 0 && !mbar_ready(&S.dfree[1], (use[1] & 1) ^ 1)) {
              nd = 1;
              d0 = step;
            } else {
              if (kc == 0) asm volatile("tcgen05.fence::after_thread_sync;");
              issue(1, kc, s);
              release(step);
            }
            if (nd >= (uint32_t)WNS || (nd > 0 && kc + 1 == nkc)) {  // ring held or group done: wait for accumulator 1
              const long long c2 = T.prof ? clock64() : 0;
              ok = wait_or_abort(&S.dfree[1], (use[1] & 1) ^ 1, abort_flag, T.wait_limit);
              if (T.prof) mw_dfree += clock64() - c2;
              if (!ok) break;
              catch_up();
            }
          } else {
            release(step);
          }
          ++step;
        }
        if (!ok) break;
        for (uint32_t g = 0; g < ng; ++g) {
          tc_commit(&S.dfull[g]);
          last_bar = &S.dfull[g];
          last_par = use[g] & 1;
          ++use[g];
        }
        ++group;
      }
      if (T.prof) {
        atomicAdd(&T.ctr->prof[2], (unsigned long long)mw_full);
        atomicAdd(&T.ctr->prof[3], (unsigned long long)mw_dfree);
        atomicAdd(&T.ctr->prof[4], (unsigned long long)(clock64() - m_start));
        atomicAdd(&T.ctr->prof[12], (unsigned long long)step);
      }
      // an aborting CTA may still have MMAs in flight: wait (bounded) for the
      // last commit, MMAs complete in issue order
      if (*abort_flag && last_bar) {
        volatile uint32_t no_abort = 0;
        wait_or_abort(last_bar, last_par, &no_abort, T.wait_limit);
      }
    }
    __syncwarp();
  } else if (warp >= WEPI0 && warp < WEPI0 + WNEPI) {
    // ============================ epilogue
    // warp w reads TMEM lane quarter w % 4 (the hardware's access rule) and
    // the 32-column blocks (w - WEPI0) / 4, + 2, + 4, ... of each accumulator
    const uint32_t quarter = warp & 3;
    const uint32_t cblk0 = (warp - WEPI0) >> 2;
    PairStage ps{pstage + (warp - WEPI0) * PSTAGE, 0, 0, P.pairs_ij != 0};
    PairStage bs{pstage + (WNEPI + warp - WEPI0) * PSTAGE, 0};
    const RingCtx rcp_{P.pair_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
    const RingCtx rcb_{P.band_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
    const RingCtx* rcp = P.ring ? &rcp_ : nullptr;
    const RingCtx* rcb = P.ring ? &rcb_ : nullptr;
    uint32_t group = 0;
    uint32_t use[WG] = {0, 0};
    bool run = true;
    long long ew = 0;
    const long long e_start = T.prof ? clock64() : 0;
    while (run) {
      const uint32_t gs = group % WGS;
      const WGroup& Gm = S.grp[gs];
      uint32_t ng = 1;
      for (uint32_t g = 0; g < ng; ++g) {
        // all lanes wait; the outcome is made warp-uniform (tcgen05.ld is .sync.aligned)
        const long long cw = T.prof ? clock64() : 0;
        const bool ok = __all_sync(FULL_MASK, wait_or_abort(&S.dfull[g], use[g] & 1, abort_flag, T.wait_limit));
        if (T.prof) ew += clock64() - cw;
        if (!ok || __any_sync(FULL_MASK, (Gm.flags & WFLAG_END) || *abort_flag)) {
          run = false;
          break;
        }
        if (g == 0) ng = Gm.ng;
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t ncols = Gm.ncols, nrows = Gm.nrows;
        const uint32_t row = g * WM + quarter * 32 + lane;  // row within the unit
        const bool row_ok = row < nrows;
        const uint32_t a_sorted = Gm.a0 + row;
        const float na = row_ok ? Gm.na[row] : 0.f;
        const uint32_t hlo = Gm.hlo, hhi = Gm.hhi, hq0 = Gm.hq0;
        // columns c in [hlo, lim) hold home rows q <= a (dropped: each pair once, no self pair)
        const uint32_t lim = (hlo < hhi && a_sorted >= hq0) ? min(hhi, hlo + min(a_sorted - hq0 + 1, (uint32_t)WN)) : 0u;
        if (g * WM + quarter * 32 < nrows) {
#pragma unroll 1
          for (uint32_t c0 = 32 * cblk0; c0 < ncols; c0 += 32 * (WNEPI / 4)) {
            uint32_t v[32];
            tmem_ld32_nowait(tbase + g * WN + ((quarter * 32u) << 16) + c0, v);
            tmem_wait();
            uint32_t o = 0;
#pragma unroll
            for (int j = 0; j < 32; j += 4) {
              const float4 h4 = *reinterpret_cast<const float4*>(&Gm.hq[c0 + j]);
              const float hv[4] = {h4.x, h4.y, h4.z, h4.w};
#pragma unroll
              for (int i = 0; i < 4; ++i) {
                const float dv = fmaf(-2.f, __uint_as_float(v[j + i]), na) + hv[i];
                v[j + i] = __float_as_uint(dv);
                o |= v[j + i];
              }
            }
            uint32_t acc_bits = 0, band_bits = 0;
            const uint32_t nvalid = min(32u, ncols - c0);
            const bool maybe = row_ok && (o >> 31);
            if (__any_sync(FULL_MASK, maybe)) {
              if (maybe) {
                uint32_t m = 0;
#pragma unroll
                for (int j = 0; j < 32; ++j) m |= (v[j] >> 31) << j;
                m &= nvalid >= 32 ? FULL_MASK : ((1u << nvalid) - 1u);
                const int e0 = (int)max(hlo, c0) - (int)c0, e1 = (int)min(lim, c0 + 32) - (int)c0;
                if (e0 < e1) m &= ~((e1 >= 32 ? FULL_MASK : ((1u << e1) - 1u)) & ~((1u << e0) - 1u));
                while (m) {
                  const int j = __ffs(m) - 1;
                  m &= m - 1;
                  if (pick32(v, j) <= -Gm.dlt[c0 + j])
                    acc_bits |= 1u << j;
                  else
                    band_bits |= 1u << j;  // decided later in FP64 (band list)
                }
              }
            }
            __syncwarp();
            const uint32_t ia = (acc_bits | band_bits) ? Gm.aid[row] : 0u;
            auto emit = [&](PairStage& stg, uint32_t bits, unsigned long long* counter, unsigned long long* list,
                            unsigned long long lcap, const RingCtx* rc) {
              stage_pairs(
                  stg, __popc(bits),
                  [&](uint32_t) {
                    const int j = __ffs(bits) - 1;
                    bits &= bits - 1;
                    const uint32_t iq = Gm.qid[c0 + j];
                    const uint32_t lo = ia < iq ? ia : iq, hi = ia < iq ? iq : ia;
                    return ((unsigned long long)lo << 32) | hi;
                  },
                  counter, list, lcap, nullptr, Gm.tag, rc);
            };
            if (__any_sync(FULL_MASK, acc_bits != 0u)) emit(ps, acc_bits, &P.ctr->pairs, P.pairs, P.cap, rcp);
            if (__any_sync(FULL_MASK, band_bits != 0u))
              emit(bs, band_bits, &P.ctr->band_n, P.band_list, P.band_cap, rcb);
          }
        }
        asm volatile("tcgen05.fence::before_thread_sync;");
        __syncwarp();
        if (lane == 0) mbar_arrive(&S.dfree[g]);
        ++use[g];
      }
      if (!run) break;
      if (lane == 0) mbar_arrive(&S.gfree[gs]);
      ++group;
    }
    stage_flush(ps, &P.ctr->pairs, P.pairs, P.cap, nullptr, rcp);
    stage_flush(bs, &P.ctr->band_n, P.band_list, P.band_cap, nullptr, rcb);
    if (T.prof && lane == 0) {
      atomicAdd(&T.ctr->prof[5], (unsigned long long)ew);
      atomicAdd(&T.ctr->prof[6], (unsigned long long)(clock64() - e_start));
    }
  }
  // all roles meet here before tensor memory is released
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == WMMA) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tbase));
  if (tid == 0 && S.abort_flag) atomicExch(&P.ctr->error, 1ull);
}

}  // namespace

namespace join {

uint32_t tcw_kd(uint32_t d, int prec) {
  const uint32_t ks = tcw_kstage(prec);
  return (d + ks - 1) / ks * ks;
}

void tcw_prepare(mistic_handle_s* h, int prec, const float* xf, uint32_t dpad32, uint32_t d, size_t n, void* xh,
                 void* xl, float* xn) {
  if (n == 0) return;
  const unsigned rows_per_block = 8;
  const unsigned grid = (unsigned)((n + rows_per_block - 1) / rows_per_block);
  if (prec == 2) {
    k_tf32_rows<<<grid, rows_per_block * 32, 0, h->stream>>>(xf, dpad32, tcw_kd(d, prec), n, (float4*)xh, xn);
    launched(h, "tf32_rows");
  } else {
    k_split_rows<<<grid, rows_per_block * 32, 0, h->stream>>>(xf, dpad32, tcw_kd(d, prec), n, (uint4*)xh,
                                                              prec == 0 ? (uint4*)xl : nullptr, xn);
    launched(h, "split_rows");
  }
}

namespace {
PFN_cuTensorMapEncodeTiled_v12000 encode_fn() {
  static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
  static std::once_flag once;
  std::call_once(once, [] {
    void* p = nullptr;
    cudaDriverEntryPointQueryResult q;
    if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) == cudaSuccess &&
        q == cudaDriverEntryPointSuccess)
      fn = (PFN_cuTensorMapEncodeTiled_v12000)p;
  });
  if (!fn) throw Error(MISTIC_ERR_CUDA, "cuTensorMapEncodeTiled is not available");
  return fn;
}

// Operand rows of kd elements, n rows; box: one stage's K x box_rows.  Split
// precision: bf16, 64-byte box rows, 64B swizzle; single bf16 or tf32:
// 128-byte box rows, 128B swizzle.
void encode_rows(CUtensorMap* m, const void* base, int prec, uint32_t kd, size_t n, uint32_t box_rows) {
  const uint32_t esz = prec == 2 ? 4 : 2;
  const cuuint64_t dims[2] = {kd, (cuuint64_t)n};
  const cuuint64_t strides[1] = {(cuuint64_t)kd * esz};
  const cuuint32_t box[2] = {tcw_kstage(prec), box_rows};
  const cuuint32_t estr[2] = {1, 1};
  const CUresult r = encode_fn()(m, prec == 2 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32 : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16, 2,
                                 const_cast<void*>(base), dims, strides, box, estr, CU_TENSOR_MAP_INTERLEAVE_NONE,
                                 prec == 0 ? CU_TENSOR_MAP_SWIZZLE_64B : CU_TENSOR_MAP_SWIZZLE_128B,
                                 CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
  if (r != CUDA_SUCCESS) throw Error(MISTIC_ERR_CUDA, "cuTensorMapEncodeTiled failed for the operand rows");
}

template <int PREC>
void launch_tcw(mistic_handle_s* h, const JoinParams& P, const TcParams& T) {
  TcwMaps maps;
  encode_rows(&maps.ah, T.xh, PREC, T.kd, T.n_rows, WM);
  if (PREC == 0)
    encode_rows(&maps.al, T.xl, PREC, T.kd, T.n_rows, WM);
  else
    maps.al = maps.ah;  // unused
  const size_t dyn = 1024 + (size_t)WNS * STAGE_BYTES + (size_t)2 * WNEPI * PSTAGE * sizeof(unsigned long long);
  MCK(cudaFuncSetAttribute(k_join_tcw<PREC>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  MCK(cudaFuncSetAttribute(k_join_tcw<PREC>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int per_sm = 0;
  MCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_join_tcw<PREC>, WTHREADS, dyn));
  if (per_sm < 1) throw Error(MISTIC_ERR_TOO_LARGE, "long-row tensor-core join does not fit on an SM");
  unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)h->sms, T.n_units);
  if (T.grid_cap) grid = std::min(grid, T.grid_cap);
  if (getenv("MISTIC_DEBUG"))
    fprintf(stderr, "[mistic] join_tcw PREC=%d KD=%u dyn=%zu occupancy=%d grid=%u units=%llu\n", PREC, T.kd, dyn,
            per_sm, grid, (unsigned long long)T.n_units);
  k_join_tcw<PREC><<<grid, WTHREADS, dyn, h->stream>>>(P, T, maps);
  launched(h, "join_tcw");
}
}  // namespace

void run_tcw(mistic_handle_s* h, const JoinParams& P, const TcParams& T) {
  if (T.n_units == 0) return;
  if (T.prec < 0 || T.prec > 2 || !T.xh || (T.prec == 0 && !T.xl) || !T.xn || T.kd == 0 ||
      T.kd % tcw_kstage(T.prec) || T.n_rows == 0)
    throw Error(MISTIC_ERR_INTERNAL, "long-row tensor-core join without prepared operand rows");
  switch (T.prec) {
    case 0: launch_tcw<0>(h, P, T); break;
    case 1: launch_tcw<1>(h, P, T); break;
    default: launch_tcw<2>(h, P, T); break;
  }
}

}  // namespace join
}  // namespace mistic
