// Tensor-core distance join (tcgen05, sm_103a).
//
// Reference counterpart: the FP64 distance loop of nodeByPoint5 /
// cachedDistanceCheck (src/kernel.cu:992-1046, 833-865).  Here a unit — up to
// 128 points of one large home bin against a segment of its neighbour bins
// (bins >= home) — is evaluated as dense 128 x 128 tiles on the 5th-generation
// tensor cores:
//
//   A row m = [a'_m, |a'_m|^2, 1, 0...]      a' = a~ - c  (c: first home row)
//   B row n = [-2 q'_n, 1, |q'_n|^2, 0...]    q' = q~ - c
//   D[m][n] = sum_k A[m][k] B[n][k] = |a'|^2 + |q'|^2 - 2 a'.q' = ||a' - q'||^2
//
// where a~, q~ are the FP32 globally centred rows.  Each operand is split
// into bf16 hi + lo parts; D = Ahi.Bhi + Ahi.Blo + Alo.Bhi is accumulated in
// FP32 in tensor memory (3 MMAs per K step of 16).  Centering at the unit's
// first row keeps |a'|, |q'| at the size of the local neighbourhood, so the
// cancellation in the Gram form stays small.
//
// Exactness: per row and tile, a rigorous bound E on |D - s64| (s64 = the
// reference FP64 predicate value) gives T_lo = eps2/(1+g64) - E and
// T_hi = eps2/(1-g64) + E: D <= T_lo accepts, D > T_hi rejects, anything in
// between is re-decided with the reference FP64 predicate.  The bound covers
//   - bf16 splitting: each product carries <= 3.02 * 2^-16 |A_k||B_k| (bf16
//     keeps 8 significant bits: |x - hi| <= 2^-8 |x|, |x - hi - lo| <= 2^-16 |x|),
//   - tensor-core FP32 accumulation: taken as <= 2^-19 per MMA instruction
//     relative to the sum of |products| (a generous allowance),
//   - FP32 norms (g_d), the FP32 centring (2uR + u(|a'|+|q'|)),
// with sum_k |A_k||B_k| <= (|a'| + |q'|)^2.  Rows whose bound exceeds
// 0.1 eps2 are re-decided entirely in FP64 (T_lo = -1, T_hi = inf).
//
// Data movement: operands are converted from the sorted FP32 rows into the
// no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core matrix;
// LBO = 128 B between K-adjacent core matrices, SBO = 16*KP B between 8-row
// groups), one elected thread issues the MMAs and commits to an mbarrier,
// and the epilogue warps read each 128 x 128 FP32 accumulator back with
// tcgen05.ld.  Every mbarrier wait is bounded; on expiry the CTA records an
// error, stops, drains its MMAs and releases its tensor memory.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "emit.cuh"
#include "internal.cuh"
#include "tc_common.cuh"

namespace mistic {
namespace {

using namespace tcu;

constexpr int TM = 128;          // home rows per tile (MMA M)
constexpr int TN = 128;          // candidate columns per tile (MMA N)
constexpr int WIN = 256;         // neighbour bins per candidate window

// ---------------------------------------------------------------- pipeline
// One persistent CTA per SM: 8 producer warps, NEPI epilogue warps, 1 MMA warp.
//   producers  fetch units; stage the unit's home rows (A: G chunks of 128,
//              once per unit) and each tile's 128 candidate rows (B) in an
//              NS-stage ring, two threads per row: raw FP32 rows arrive by
//              cp.async (in a RAW-slot landing ring, or in the B stage
//              itself) and are converted in place into bf16 hi/lo with the
//              per-column threshold folded into B (column d+1 holds
//              |q'|^2 - T(n)); up to LA tiles are in flight;
//   MMA warp   one lane issues 3 * KP/16 tcgen05.mma per (tile, home chunk)
//              into the next of NACC = 4 TMEM accumulators and commits;
//   epilogue   tcgen05.ld of TMEM lane quarter w % 4, sign-bit test (D' < 0
//              marks a candidate), home-bin rule by column range, sure
//              accepts to the pair list, the error band to the band list.
// Barriers (all waits bounded by a %globaltimer deadline):
//   full[s]   producers -> MMA        (NPROD arrivals)
//   sfree[s]  epilogue  -> producers  (NEPI arrivals after the tile's last home chunk)
//   dfull[b]  MMA       -> epilogue   (tcgen05.commit, or a plain arrive on the terminate tile)
//   dfree[b]  epilogue  -> MMA        (NEPI arrivals; accumulator b reusable)
//   afull     producers -> MMA        (NPROD arrivals per unit: A written)
//   afree     MMA       -> producers  (tcgen05.commit after a unit's last tile)
constexpr int NPW = 8;     // producer warps: two threads per operand row
constexpr int NPROD = NPW * 32;
// NEPI epilogue warps (a template parameter: 8 or 16) cover the 4 TMEM lane
// quarters x NEPI / 4 column-block groups; the MMA warp follows them.
constexpr int EPI0 = NPW;  // first epilogue warp (a multiple of 4: warp % 4 is its lane quarter)
__host__ __device__ constexpr int tc_threads(int nepi) { return (EPI0 + nepi + 1) * 32; }
constexpr int NACC = 4;    // TMEM accumulators of 128 columns (512 per CTA, one CTA per SM)
constexpr uint32_t FLAG_FIRST = 1, FLAG_LAST = 2, FLAG_END = 4;

struct TileMeta {
  uint32_t a0, na, ncols, flags, ng;  // ng: 128-row MMA tiles of this unit (1..G)
  uint32_t hcr, hq;  // columns [hcr & 255, hcr >> 8) hold home-bin rows, the first at sorted position hq
  uint32_t inst;     // instance of the unit (fused batch joins; else 0)
};

template <int NS, int G, int RAW>
struct TcShared2 {
  __align__(16) float cadd_a[128];  // -c   (A rows: x - c)
  __align__(16) float cadd_b[128];  // 2c   (B rows: -2 (x - c))
  uint32_t w_home;  // (window generation << 8) | index of the home bin in the window
  uint32_t hx[4][2];  // home column range of issued tiles (producer thread 0 only)
  uint32_t qid[NS][TN];      // original row ids of the candidates
  uint32_t aid[NS][TM * G];  // original row ids of the home rows (per stage: the epilogue
                             // may still read a finished unit while producers start the next)
  float dlt[NS][TN];  // accept when D' <= -dlt
  TileMeta meta[NS];
  uint32_t rid[RAW > 0 ? RAW : 1][TN];  // candidate ids of the tiles in the raw ring
  uint32_t w_start[WIN];
  uint32_t w_pref[WIN + 1];
  uint32_t scan_ws[NPW];
  unsigned long long unit;
  uint32_t w_total, w_pos, seg_next, w_nb;
  uint32_t ra2max;  // float bits, non-negative
  uint32_t abort_flag;
  uint32_t tmem_base;
  uint32_t pflag[2];  // producer-wide decisions, written by producer thread 0
  // [tile parity][K-block parity][row]: partial row norms of the two threads
  // of a row (two-threads-a-row mode only; pair mode has one thread a row)
  float npart[RAW == 4 ? 1 : 2][2][RAW == 4 ? 1 : TM];
  unsigned long long full[NS], sfree[NS], dfull[NACC], dfree[NACC], afull, afree;
};

__device__ __forceinline__ void prod_sync() { asm volatile("bar.sync 1, %0;" ::"n"(NPROD) : "memory"); }

// Operand rows live in the no-swizzle K-major core-matrix layout: the
// 16-byte chunk of row r and K block kb (8 bf16) sits at bf16 offset
// chunk_off(r, kb).  A raw FP32 row is first copied (cp.async) into the
// chunk slots of the row itself -- floats [8kb, 8kb+4) into the hi chunk of
// block kb, [8kb+4, 8kb+8) into its lo chunk -- and then converted in place,
// block by block, into the augmented bf16 hi/lo row.  Two threads share a
// row, one per parity of the K blocks (kb = 2j + half); a thread only touches
// its own chunks.  Blocks wholly beyond the augmented columns (k0 >= d + 2)
// are cleared once when the kernel starts and never written again.
template <int KP>
__device__ __forceinline__ void load_half(__nv_bfloat16* hi, __nv_bfloat16* lo, uint32_t r, uint32_t half,
                                          const float* __restrict__ xr, uint32_t dpad) {
  constexpr int HB = KP / 16;
#pragma unroll
  for (int j = 0; j < HB; ++j) {
    const uint32_t kb = 2 * j + half, k0 = 8 * kb, off = chunk_off<KP>(r, kb);
    if (k0 < dpad) cp_async16(hi + off, xr + k0);
    if (k0 + 4 < dpad) cp_async16(lo + off, xr + k0 + 4);
  }
}

__device__ __forceinline__ void unpack8(const __nv_bfloat16* hi, const __nv_bfloat16* lo, uint32_t off, bool l0,
                                        bool l1, float (&x)[8]) {
  float4 x0 = make_float4(0.f, 0.f, 0.f, 0.f), x1 = x0;
  if (l0) x0 = *reinterpret_cast<const float4*>(hi + off);
  if (l1) x1 = *reinterpret_cast<const float4*>(lo + off);
  x[0] = x0.x, x[1] = x0.y, x[2] = x0.z, x[3] = x0.w;
  x[4] = x1.x, x[5] = x1.y, x[6] = x1.z, x[7] = x1.w;
}

__device__ __forceinline__ void store_split(__nv_bfloat16* hi, __nv_bfloat16* lo, uint32_t off, const float (&v)[8]) {
  uint4 oh, ol;
  uint32_t* ph = reinterpret_cast<uint32_t*>(&oh);
  uint32_t* pl = reinterpret_cast<uint32_t*>(&ol);
#pragma unroll
  for (int i = 0; i < 4; ++i) {
    const __nv_bfloat162 hv = __floats2bfloat162_rn(v[2 * i], v[2 * i + 1]);
    const float2 hf = __bfloat1622float2(hv);
    const __nv_bfloat162 lv = __floats2bfloat162_rn(v[2 * i] - hf.x, v[2 * i + 1] - hf.y);
    ph[i] = *reinterpret_cast<const uint32_t*>(&hv);
    pl[i] = *reinterpret_cast<const uint32_t*>(&lv);
  }
  *reinterpret_cast<uint4*>(hi + off) = oh;
  *reinterpret_cast<uint4*>(lo + off) = ol;
}

// Operand values: scale * fl(x[k] - c[k]) = fma(x[k], scale, cadd[k]) with
// cadd = -scale * c, exactly (scale is 1 or -2).  The row norm |x - c|^2 is
// accumulated from the scaled values (fma(v, v, acc) = scale^2 fma(t, t, acc')
// exactly) in K order per half; the halves are added by the caller.
//
// Pass 1 writes every K block of this thread that holds a data or an
// augmented column, with placeholders pd, pd1 in the augmented columns d and
// d + 1, and returns the partial sum of v^2; once the two halves of the norm
// are added, patch_col writes the one augmented value that depends on it
// (|a'|^2 in column d of A, |q'|^2 - T in column d + 1 of B).  A block is
// read before it is written, so the source may be the destination.
template <int KP>
__device__ __forceinline__ float conv_pass1(const __nv_bfloat16* sh, const __nv_bfloat16* sl, __nv_bfloat16* hi,
                                            __nv_bfloat16* lo, uint32_t r, uint32_t half, bool ok, const float* cadd,
                                            float scale, uint32_t d, float pd, float pd1) {
  constexpr int HB = KP / 16;
  float acc = 0.f;
  if (!ok) return acc;  // a column beyond the tile: its stale values are masked by the epilogue
#pragma unroll 2
  for (int j = 0; j < HB; ++j) {
    const uint32_t kb = 2 * j + half, k0 = 8 * kb, off = chunk_off<KP>(r, kb);
    float v[8];
    if (k0 >= d + 2) continue;  // zero block (cleared at the start)
    float x[8];
    unpack8(sh, sl, off, k0 < d, k0 + 4 < d, x);
    if (k0 + 8 <= d) {  // full block
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        v[i] = fmaf(x[i], scale, cadd[k0 + i]);
        acc = fmaf(v[i], v[i], acc);
      }
    } else {  // holds d or d + 1
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const uint32_t k = k0 + i;
        float t = 0.f;
        if (k < d) {
          t = fmaf(x[i], scale, cadd[k]);
          acc = fmaf(t, t, acc);
        } else if (k == d) {
          t = pd;
        } else if (k == d + 1) {
          t = pd1;
        }
        v[i] = t;
      }
    }
    store_split(hi, lo, off, v);
  }
  return acc;
}

// Whole-row forms for one thread a row (pair mode): the raw row's chunks
// land in the row's own slots as in load_half, every K block of the row.
template <int KP>
__device__ __forceinline__ void load_row(__nv_bfloat16* hi, __nv_bfloat16* lo, uint32_t r,
                                         const float* __restrict__ xr, uint32_t dpad) {
#pragma unroll
  for (int kb = 0; kb < KP / 8; ++kb) {
    const uint32_t k0 = 8 * kb, off = chunk_off<KP>(r, kb);
    if (k0 < dpad) cp_async16(hi + off, xr + k0);
    if (k0 + 4 < dpad) cp_async16(lo + off, xr + k0 + 4);
  }
}

// Converts row r from the raw chunks (sh, sl) into the bf16 hi/lo operand row
// (hi, lo), K blocks in order, with placeholders pd, pd1 in the augmented
// columns d and d + 1; returns the row norm |x - c|^2 (times scale^2).
template <int KP>
__device__ __forceinline__ float conv_row(const __nv_bfloat16* sh, const __nv_bfloat16* sl, __nv_bfloat16* hi,
                                          __nv_bfloat16* lo, uint32_t r, const float* cadd, float scale, uint32_t d,
                                          float pd, float pd1) {
  float acc = 0.f;
#pragma unroll
  for (int kb = 0; kb < KP / 8; ++kb) {
    const uint32_t k0 = 8 * kb, off = chunk_off<KP>(r, kb);
    if (k0 >= d + 2) break;  // zero blocks (cleared at the start)
    float x[8], v[8];
    unpack8(sh, sl, off, k0 < d, k0 + 4 < d, x);
    if (k0 + 8 <= d) {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        v[i] = fmaf(x[i], scale, cadd[k0 + i]);
        acc = fmaf(v[i], v[i], acc);
      }
    } else {
#pragma unroll
      for (int i = 0; i < 8; ++i) {
        const uint32_t k = k0 + i;
        float t = 0.f;
        if (k < d) {
          t = fmaf(x[i], scale, cadd[k]);
          acc = fmaf(t, t, acc);
        } else if (k == d) {
          t = pd;
        } else if (k == d + 1) {
          t = pd1;
        }
        v[i] = t;
      }
    }
    store_split(hi, lo, off, v);
  }
  return acc;
}

// Column k of row r := v, split into bf16 hi + lo as store_split does.
template <int KP>
__device__ __forceinline__ void patch_col(__nv_bfloat16* hi, __nv_bfloat16* lo, uint32_t r, uint32_t k, float v) {
  const uint32_t off = chunk_off<KP>(r, k >> 3) + (k & 7);
  const __nv_bfloat16 h = __float2bfloat16_rn(v);
  hi[off] = h;
  lo[off] = __float2bfloat16_rn(v - __bfloat162float(h));
}

template <int KP, int NS, int G, int RAW, int NEPI>
__global__ void __launch_bounds__(tc_threads(NEPI), 1) k_join_tc(const JoinParams P, const TcParams T) {
  constexpr int MMA_WARP = EPI0 + NEPI;
  extern __shared__ __align__(128) unsigned char tc_dyn[];
  __shared__ TcShared2<NS, G, RAW> S;
  constexpr uint32_t OPB = TM * KP;  // bf16 elements per operand buffer
  __nv_bfloat16* Ahi = reinterpret_cast<__nv_bfloat16*>(tc_dyn);  // G home chunks of 128 rows
  __nv_bfloat16* Alo = Ahi + G * OPB;
  __nv_bfloat16* Bhi = Alo + G * OPB;  // NS stages of hi, then NS stages of lo
  __nv_bfloat16* Blo = Bhi + NS * OPB;
  __nv_bfloat16* Raw = Blo + NS * OPB;  // RAW landing slots (raw FP32 rows in the chunk layout, 2 * OPB each)
  unsigned long long* pstage = reinterpret_cast<unsigned long long*>(Raw + RAW * 2 * OPB);  // 2 NEPI x PSTAGE
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  volatile uint32_t* abort_flag = &S.abort_flag;

  if (tid == 0) {
    for (int i = 0; i < NS; ++i) {
      mbar_init(&S.full[i], RAW == 4 ? TM : NPROD);  // pair mode: one group of 128 a tile
      mbar_init(&S.sfree[i], NEPI);
    }
    for (int i = 0; i < NACC; ++i) {
      mbar_init(&S.dfull[i], 1);
      mbar_init(&S.dfree[i], NEPI);
    }
    mbar_init(&S.afull, NPROD);
    mbar_init(&S.afree, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    S.abort_flag = 0;
    S.w_home = 0xffffffffu;
  }
  if (warp == MMA_WARP) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 512;" ::"r"(smem_u32(&S.tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  {  // operand buffers start at zero: K blocks beyond the augmented columns are never written
    uint4* z = reinterpret_cast<uint4*>(tc_dyn);
    const uint32_t nz = (2 * G + 2 * NS) * OPB * (uint32_t)sizeof(__nv_bfloat16) / 16;
    for (uint32_t i = tid; i < nz; i += blockDim.x) z[i] = make_uint4(0u, 0u, 0u, 0u);
    asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = S.tmem_base;

  if (warp < NPW) {
    if constexpr (RAW == 4) {
    // ============================ producers, pair mode (K <= 32, four raw slots)
    // The 256 producer threads are two groups of 128; thread (grp, pr)
    // converts the whole row pr of one candidate tile, group grp of each
    // pair of consecutive tiles, so a row needs no exchange and its fixed
    // costs (finding its source row, issuing its copies, its threshold and
    // metadata) are paid once.  Pairs never span a window of neighbour bins:
    // when fewer than 129 candidate ranks are left in it, the pair is one
    // tile and group 1 idles.  Two pairs are in flight, the one being
    // converted and the next (one raw slot a tile).  Branches that lead to bar.sync depend only on values every
    // producer thread holds or reads after the same bar.sync; barrier waits
    // are done by thread 0 and broadcast through S.pflag.
    const uint32_t pr = (uint32_t)tid & 127u, grp = (uint32_t)tid >> 7;
    uint32_t tile = 0, issued = 0, unit_k = 0, pf = 0;
    unsigned long long n_tiles = 0, n_cells = 0;
    long long pw_sfree = 0, pc_unit = 0, pc_win = 0, pc_conv = 0, pc_ldw = 0;
    long long pc_adv = 0, pc_bar = 0, pc_p1 = 0, pc_p2 = 0, pc_fin = 0;
    uint32_t wgen = 0;
    const long long p_start = T.prof ? clock64() : 0;
    auto end_marker = [&]() {  // next tile slot: tells the MMA warp and the epilogue to stop
      const uint32_t st = tile % NS;
      if (tid == 0) {
        wait_or_abort(&S.sfree[st], ((tile / NS) & 1) ^ 1, abort_flag, T.wait_limit);
        S.meta[st].flags = FLAG_END;
      }
      prod_sync();
      if (grp == 0) mbar_arrive(&S.full[st]);
    };
    for (;;) {
      const long long cu0 = T.prof ? clock64() : 0;
      const uint32_t slot = pf++ & 1;
      if (tid == 0) {
        const unsigned long long t = atomicAdd(&T.ctr->next_unit, 1ull);
        const unsigned long long uu = t < T.n_def_in ? (unsigned long long)T.def_in[t] : T.main_start + (t - T.n_def_in);
        S.unit = uu;
        bool go = (T.claim_cap == 0 || t < T.claim_cap) && uu < T.n_units && !*abort_flag;
        if (go && P.ring && *(volatile unsigned long long*)&P.ctr->stop) {
          const RingCtx rc{P.pair_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
          ring_defer(&rc, P.tag_base_tc + (uint32_t)uu);
          go = false;
        }
        if (go && unit_k > 0) go = wait_or_abort(&S.afree, (unit_k - 1) & 1, abort_flag, T.wait_limit);
        S.pflag[slot] = go ? 1u : 0u;
      }
      prod_sync();
      if (!S.pflag[slot]) {
        end_marker();
        break;
      }
      const unsigned long long u = S.unit;
      const Unit U = T.units[u];
      const float* X = (const float*)P.xs;
      const uint32_t *bstart = P.bstart, *nbr = P.nbr, *ids = P.ids;
      TcBound tb = T.b;
      uint32_t inst = 0;
      if (T.unit_inst) {
        inst = T.unit_inst[u];
        const InstDesc& I = P.insts[inst];
        X = (const float*)I.xs;
        bstart = I.bstart;
        nbr = I.nbr;
        ids = I.ids;
        tb = I.tcb;
      }
      if (P.ring) inst = P.tag_base_tc + (uint32_t)u;
      const uint32_t hs = bstart[U.h], he = bstart[U.h + 1];
      const uint32_t a0 = hs + U.chunk * (TM * G);
      const uint32_t na = min((uint32_t)(TM * G), he - a0);
      const uint32_t ng = (na + TM - 1) / TM;
      if (tid < (int)P.dpad) {
        const float c = X[(size_t)a0 * P.dpad + tid];
        S.cadd_a[tid] = -c;
        S.cadd_b[tid] = 2.f * c;
      }
      if (tid == 0) S.ra2max = 0;
      prod_sync();
      uint32_t my_aid[G];  // original ids of home rows g * TM + pr
#pragma unroll
      for (int g = 0; g < G; ++g) {
        const uint32_t r = g * TM + pr;
        my_aid[g] = r < na ? ids[a0 + r] : 0u;
      }
      {  // home rows r = tid + 256 i, whole rows
        constexpr int HR = (G * TM + NPROD - 1) / NPROD;
#pragma unroll
        for (int i = 0; i < HR; ++i) {
          const uint32_t r = (uint32_t)tid + NPROD * i;
          if (r < na)
            load_row<KP>(Ahi + (r / TM) * OPB, Alo + (r / TM) * OPB, r % TM, X + (size_t)(a0 + r) * P.dpad, P.dpad);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        float m = 0.f;
#pragma unroll
        for (int i = 0; i < HR; ++i) {
          const uint32_t r = (uint32_t)tid + NPROD * i;
          if (r < na) {
            __nv_bfloat16 *ah = Ahi + (r / TM) * OPB, *al = Alo + (r / TM) * OPB;
            const float nrm = conv_row<KP>(ah, al, ah, al, r % TM, S.cadd_a, 1.f, P.d, 0.f, 1.f);
            patch_col<KP>(ah, al, r % TM, P.d, nrm);
            m = fmaxf(m, nrm);
          }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL_MASK, m, o));
        if (lane == 0) atomicMax(&S.ra2max, __float_as_uint(m));
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&S.afull);
      prod_sync();
      const float ra2max = __uint_as_float(S.ra2max);
      if (T.prof) pc_unit += clock64() - cu0;

      // ---- candidate pairs of tiles of this unit
      uint32_t seg_next = U.s0, w_nb = 0, w_pos = 0, w_total = 0;
      unsigned long long pq = 0;  // per pair in flight: colsA | lastA << 8 | colsB << 9 | lastB << 17
      uint32_t pin = 0;           // pairs in flight
      int w_hj = -1;
      auto home_cols = [&](uint32_t pos, uint32_t ncols, uint32_t* hcr, uint32_t* hq) {
        *hcr = 0;
        *hq = 0;
        if (w_hj >= 0 && ncols > 0) {
          const uint32_t hr0 = S.w_pref[w_hj], hr1 = S.w_pref[w_hj + 1];
          if (max(hr0, pos) < min(hr1, pos + ncols)) {
            const uint32_t lo = max(hr0, pos) - pos, hi = min(hr1, pos + ncols) - pos;
            *hcr = lo | (hi << 8);
            *hq = hs + (pos + lo - hr0);
          }
        }
      };
      // issues the next pair: returns 1, or 2 on abort
      auto advance = [&]() -> int {
        while (w_pos >= w_total) {
          const long long cw0 = T.prof ? clock64() : 0;
          const uint32_t nb = min((uint32_t)WIN, U.s1 - seg_next);
          uint32_t st0 = 0, sz0 = 0, bn = 0xffffffffu;
          if ((uint32_t)tid < nb) {
            bn = nbr[seg_next + tid];
            st0 = bstart[bn];
            sz0 = bstart[bn + 1] - st0;
          }
          const uint32_t incl = warp_scan_incl(sz0);
          if (lane == 31) S.scan_ws[warp] = incl;
          prod_sync();
          uint32_t wp = 0;
          for (int w = 0; w < warp; ++w) wp += S.scan_ws[w];
          ++wgen;
          if ((uint32_t)tid < nb) {
            S.w_start[tid] = st0;
            S.w_pref[tid + 1] = wp + incl;
            if (bn == U.h) S.w_home = ((wgen & 0xffffffu) << 8) | (uint32_t)tid;
          }
          if (tid == 0) S.w_pref[0] = 0;
          prod_sync();
          {
            const uint32_t wh = S.w_home;
            w_hj = (wh >> 8) == (wgen & 0xffffffu) ? (int)(wh & 255u) : -1;
          }
          w_nb = nb;
          w_pos = 0;
          w_total = S.w_pref[nb];
          seg_next += nb;
          if (T.prof) pc_win += clock64() - cw0;
        }
        const long long ca0 = T.prof ? clock64() : 0;
        const uint32_t left = w_total - w_pos;
        const uint32_t colsA = min((uint32_t)TN, left);
        const uint32_t colsB = left > (uint32_t)TN ? min((uint32_t)TN, left - TN) : 0u;
        const bool more = seg_next < U.s1;  // further windows after this one
        const bool lastA = colsB == 0 && left <= (uint32_t)TN && !more;
        const bool lastB = colsB > 0 && left <= 2u * TN && !more;
        const uint32_t mycols = grp ? colsB : colsA;
        // row of candidate rank w_pos + tid (warp-wide probes of the window prefix)
        uint32_t q = 0xffffffffu;
        {
          const uint32_t r0 = w_pos + ((uint32_t)tid & ~31u);
          const uint32_t step = (w_nb + 31) >> 5;
          const uint32_t c = __popc(__ballot_sync(FULL_MASK, lane * step < w_nb && S.w_pref[lane * step] <= r0));
          const uint32_t base = (c - 1) * step;
          const uint32_t b0 =
              base + __popc(__ballot_sync(FULL_MASK, (uint32_t)lane < step && base + lane < w_nb &&
                                                         S.w_pref[base + lane] <= r0)) - 1;
          const uint32_t e = b0 + 1 + lane;
          const uint32_t t = e <= w_nb ? S.w_pref[e] - r0 : 32u;
          const uint32_t bounds = __reduce_or_sync(FULL_MASK, t < 32u ? 1u << t : 0u);
          if (pr < mycols) {
            const uint32_t b = b0 + __popc(bounds & ((2u << lane) - 1u));
            q = S.w_start[b] + (r0 + lane - S.w_pref[b]);
          }
        }
        const uint32_t rs = (issued + grp) % RAW;
        __nv_bfloat16* dh = Raw + rs * 2 * OPB;
        __nv_bfloat16* dl = dh + OPB;
        if (pr < mycols) {
          asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(&S.rid[rs][pr])), "l"(ids + q)
                       : "memory");
          load_row<KP>(dh, dl, pr, X + (size_t)q * P.dpad, P.dpad);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        if (tid == 0) {
          uint32_t hcr, hq;
          home_cols(w_pos, colsA, &hcr, &hq);
          S.hx[issued & 3][0] = hcr;
          S.hx[issued & 3][1] = hq;
          home_cols(w_pos + TN, colsB, &hcr, &hq);
          S.hx[(issued + 1) & 3][0] = hcr;
          S.hx[(issued + 1) & 3][1] = hq;
        }
        pq |= (unsigned long long)(colsA | (lastA ? 0x100u : 0u) | (colsB << 9) | (lastB ? 0x20000u : 0u))
              << (18 * pin);
        ++pin;
        w_pos += colsB > 0 ? 2u * TN : (uint32_t)TN;
        issued += colsB > 0 ? 2u : 1u;
        if (T.prof) pc_adv += clock64() - ca0;
        return 1;
      };

      // One pair is in flight ahead of the pair being converted.  The next
      // pair's copies and home-column entries are issued only after the
      // barrier that ends every thread's work on the pair before it, whose
      // raw slots and entries they reuse: a pair of one tile shifts the slots
      // by one, so the thread that converted a slot is not always the thread
      // that refills it.
      bool first = true, aborted = false;
      if (w_pos < w_total || seg_next < U.s1) advance();
      for (;;) {
        if (pin == 0) break;
        const long long cc0 = T.prof ? clock64() : 0;
        asm volatile("cp.async.wait_group 0;" ::: "memory");
        if (T.prof) pc_ldw += clock64() - cc0;
        const uint32_t e = (uint32_t)(pq & 0x3ffffull);
        pq >>= 18;
        --pin;
        const uint32_t colsA = e & 0xffu, colsB = (e >> 9) & 0xffu;
        const bool lastA = (e & 0x100u) != 0u, lastB = (e & 0x20000u) != 0u;
        const uint32_t nt = colsB > 0 ? 2u : 1u;
        const long long cb0 = T.prof ? clock64() : 0;
        const uint32_t fl = pf++ & 1;
        if (tid == 0) {
          const long long c0 = T.prof ? clock64() : 0;
          bool ok = wait_or_abort(&S.sfree[tile % NS], ((tile / NS) & 1) ^ 1, abort_flag, T.wait_limit);
          if (ok && nt == 2)
            ok = wait_or_abort(&S.sfree[(tile + 1) % NS], (((tile + 1) / NS) & 1) ^ 1, abort_flag, T.wait_limit);
          S.pflag[fl] = ok ? 1u : 0u;
          if (T.prof) pw_sfree += clock64() - c0;
        }
        prod_sync();
        if (T.prof) pc_bar += clock64() - cb0;
        if (!S.pflag[fl]) {
          aborted = true;
          break;
        }
        if (w_pos < w_total || seg_next < U.s1) advance();
        if (grp < nt) {
          const uint32_t mt = tile + grp;
          const uint32_t st = mt % NS, rs = mt % RAW;
          const uint32_t ncols = grp ? colsB : colsA;
          const bool last = grp ? lastB : lastA;
          const bool ok = pr < ncols;
          __nv_bfloat16* bh = Bhi + st * OPB;
          __nv_bfloat16* bl = Blo + st * OPB;
          const long long cp0 = T.prof ? clock64() : 0;
          if (ok) {
            const __nv_bfloat16* sh = Raw + rs * 2 * OPB;
            S.qid[st][pr] = S.rid[rs][pr];
            const float nq2 = conv_row<KP>(sh, sh + OPB, bh, bl, pr, S.cadd_b, -2.f, P.d, 1.f, 0.f) * 0.25f;
            float tcol = 0.f, dl = 0.f;
            if (!column_threshold(tb, ra2max, nq2, &tcol, &dl)) {
              tcol = 1e30f;   // every row of this column becomes a candidate ...
              dl = INFINITY;  // ... and none is accepted without the FP64 check
            }
            patch_col<KP>(bh, bl, pr, P.d + 1, nq2 - tcol);
            S.dlt[st][pr] = dl;
          }
          const long long cp1 = T.prof ? clock64() : 0;
#pragma unroll
          for (int g = 0; g < G; ++g) S.aid[st][g * TM + pr] = my_aid[g];
          if (pr == 0) {
            S.meta[st] = TileMeta{a0, na, ncols, (first && grp == 0 ? FLAG_FIRST : 0u) | (last ? FLAG_LAST : 0u), ng,
                                  S.hx[mt & 3][0], S.hx[mt & 3][1], inst};
            n_tiles += 1;
            n_cells += (unsigned long long)na * ncols;
          }
          asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
          mbar_arrive(&S.full[st]);
          if (T.prof) {
            const long long ce = clock64();
            pc_p1 += cp1 - cp0;
            pc_fin += ce - cp1;
            pc_conv += ce - cc0;
          }
        }
        first = false;
        tile += nt;
      }
      asm volatile("cp.async.wait_all;" ::: "memory");
      ++unit_k;
      if (aborted) {
        end_marker();
        break;
      }
    }
    if (pr == 0 && n_tiles) {
      atomicAdd(&T.ctr->tiles, n_tiles);
      atomicAdd(&T.ctr->cells, n_cells);
    }
    if (tid == 0 && T.prof) {
      atomicAdd(&T.ctr->prof[0], (unsigned long long)pw_sfree);
      atomicAdd(&T.ctr->prof[1], (unsigned long long)(clock64() - p_start));
      atomicAdd(&T.ctr->prof[7], (unsigned long long)pc_unit);
      atomicAdd(&T.ctr->prof[8], (unsigned long long)pc_win);
      atomicAdd(&T.ctr->prof[9], (unsigned long long)pc_conv);
      atomicAdd(&T.ctr->prof[14], (unsigned long long)pc_ldw);
      atomicAdd(&T.ctr->prof[16], (unsigned long long)pc_adv);
      atomicAdd(&T.ctr->prof[17], (unsigned long long)pc_bar);
      atomicAdd(&T.ctr->prof[18], (unsigned long long)pc_p1);
      atomicAdd(&T.ctr->prof[19], (unsigned long long)pc_p2);
      atomicAdd(&T.ctr->prof[20], (unsigned long long)pc_fin);
    }
    } else {
    // ============================ producers (NPW warps, two threads per row)
    // Thread (prow, half): row prow = 32 * (warp % 4) + lane of every operand
    // tile, K blocks kb = 2j + half with half = warp / 4, so the lanes of a
    // warp take the same branches; the two halves of a row norm meet in
    // S.npart (one bar.sync).  Every branch that
    // leads to bar.sync is taken on a value all producer threads hold in
    // registers or read from shared memory after the same bar.sync; barrier
    // waits are done by thread 0 and broadcast through S.pflag[2] (two slots:
    // a thread is at most one bar.sync behind thread 0).
    const uint32_t prow = ((uint32_t)(warp & 3) << 5) | (uint32_t)lane, half = (uint32_t)warp >> 2;
    uint32_t xpar = 0;  // parity of the next S.npart exchange
    // row norm from this thread's part and the other half's (all producer
    // threads call it together)
    auto row_norm = [&](float part) {
      S.npart[xpar][half][prow] = part;
      prod_sync();
      const float o = S.npart[xpar][half ^ 1][prow];
      xpar ^= 1;
      return half == 0 ? part + o : o + part;  // the same sum, in the same order, in both threads
    };
    uint32_t tile = 0, issued = 0, unit_k = 0, pf = 0;
    unsigned long long n_tiles = 0, n_cells = 0;
    long long pw_sfree = 0, pc_unit = 0, pc_win = 0, pc_conv = 0, pc_ldw = 0;
    long long pc_adv = 0, pc_bar = 0, pc_p1 = 0, pc_p2 = 0, pc_fin = 0;
    uint32_t wgen = 0;  // window refills so far (tags S.w_home)
    // tiles in flight: RAW landing slots, or (rows landing in the B stages
    // themselves) NS - 1, so that issuing tile t + LA - 1 waits only on tiles
    // before t
    constexpr uint32_t LA = RAW > 0 ? RAW : (NS - 1 < 3 ? NS - 1 : 3);
    const long long p_start = T.prof ? clock64() : 0;
    auto end_marker = [&]() {  // last tile slot: tells the MMA warp and the epilogue to stop
      const uint32_t st = tile % NS;
      if (tid == 0) {
        wait_or_abort(&S.sfree[st], ((tile / NS) & 1) ^ 1, abort_flag, T.wait_limit);
        S.meta[st].flags = FLAG_END;
      }
      prod_sync();
      mbar_arrive(&S.full[st]);
    };
    for (;;) {
      const long long cu0 = T.prof ? clock64() : 0;
      const uint32_t slot = pf++ & 1;
      if (tid == 0) {
        // claim index -> unit: units deferred by the last ring pass first,
        // then the list from main_start (the identity outside ring mode)
        const unsigned long long t = atomicAdd(&T.ctr->next_unit, 1ull);
        const unsigned long long uu = t < T.n_def_in ? (unsigned long long)T.def_in[t] : T.main_start + (t - T.n_def_in);
        S.unit = uu;
        bool go = (T.claim_cap == 0 || t < T.claim_cap) && uu < T.n_units && !*abort_flag;
        if (go && P.ring && *(volatile unsigned long long*)&P.ctr->stop) {  // the ring filled: leave it for the next pass
          const RingCtx rc{P.pair_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
          ring_defer(&rc, P.tag_base_tc + (uint32_t)uu);
          go = false;
        }
        if (go && unit_k > 0) go = wait_or_abort(&S.afree, (unit_k - 1) & 1, abort_flag, T.wait_limit);  // A no longer read
        S.pflag[slot] = go ? 1u : 0u;
      }
      prod_sync();
      if (!S.pflag[slot]) {
        end_marker();
        break;
      }
      const unsigned long long u = S.unit;
      const Unit U = T.units[u];
      // the unit's instance: its arrays and bound constants (fused batch
      // joins), or the launch's own
      const float* X = (const float*)P.xs;
      const uint32_t *bstart = P.bstart, *nbr = P.nbr, *ids = P.ids;
      TcBound tb = T.b;
      uint32_t inst = 0;
      if (T.unit_inst) {
        inst = T.unit_inst[u];
        const InstDesc& I = P.insts[inst];
        X = (const float*)I.xs;
        bstart = I.bstart;
        nbr = I.nbr;
        ids = I.ids;
        tb = I.tcb;
      }
      if (P.ring) inst = P.tag_base_tc + (uint32_t)u;  // the ring's tag of this unit's pairs
      const uint32_t hs = bstart[U.h], he = bstart[U.h + 1];
      const uint32_t a0 = hs + U.chunk * (TM * G);
      const uint32_t na = min((uint32_t)(TM * G), he - a0);
      const uint32_t ng = (na + TM - 1) / TM;
      if (tid < (int)P.dpad) {
        const float c = X[(size_t)a0 * P.dpad + tid];
        S.cadd_a[tid] = -c;
        S.cadd_b[tid] = 2.f * c;
      }
      if (tid == 0) S.ra2max = 0;
      prod_sync();
      uint32_t my_aid[(G + 1) / 2];  // original ids of home rows g * TM + prow, g = half, half + 2, ...
#pragma unroll
      for (int i = 0; i < (G + 1) / 2; ++i) {
        const uint32_t r = (2 * i + half) * TM + prow;
        my_aid[i] = (2 * i + (int)half < G && r < na) ? ids[a0 + r] : 0u;
      }
      {
        for (uint32_t g = 0; g < ng; ++g) {
          const uint32_t r = g * TM + prow;
          if (r < na) load_half<KP>(Ahi + g * OPB, Alo + g * OPB, prow, half, X + (size_t)(a0 + r) * P.dpad, P.dpad);
        }
        asm volatile("cp.async.wait_all;" ::: "memory");
        float m = 0.f;
        for (uint32_t g = 0; g < ng; ++g) {
          const bool ok = g * TM + prow < na;
          __nv_bfloat16 *ah = Ahi + g * OPB, *al = Alo + g * OPB;
          const float part = conv_pass1<KP>(ah, al, ah, al, prow, half, ok, S.cadd_a, 1.f, P.d, 0.f, 1.f);
          const float nrm = row_norm(part);
          if (ok && ((P.d >> 3) & 1u) == half) patch_col<KP>(ah, al, prow, P.d, nrm);
          m = fmaxf(m, ok ? nrm : 0.f);
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL_MASK, m, o));
        if (lane == 0) atomicMax(&S.ra2max, __float_as_uint(m));
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&S.afull);
      prod_sync();
      const float ra2max = __uint_as_float(S.ra2max);
      if (T.prof) pc_unit += clock64() - cu0;

      // ---- candidate tiles of this unit: window of up to WIN neighbour bins
      // (state uniform, in registers); the rows of up to LA tiles are in
      // flight (cp.async, one group per tile) while the oldest is converted
      uint32_t seg_next = U.s0, w_nb = 0, w_pos = 0, w_total = 0;
      uint32_t pq = 0;  // (columns | last << 8) of the tiles in flight, 9 bits each, oldest lowest
      int w_hj = -1;    // index of the home bin in the window, or -1
      // 1: tile issued; 2: abort
      auto advance = [&]() -> int {
        while (w_pos >= w_total) {  // the caller checked that the unit has more tiles
          const long long cw0 = T.prof ? clock64() : 0;
          const uint32_t nb = min((uint32_t)WIN, U.s1 - seg_next);
          uint32_t st0 = 0, sz0 = 0, bn = 0xffffffffu;
          if ((uint32_t)tid < nb) {
            bn = nbr[seg_next + tid];
            st0 = bstart[bn];
            sz0 = bstart[bn + 1] - st0;
          }
          const uint32_t incl = warp_scan_incl(sz0);
          if (lane == 31) S.scan_ws[warp] = incl;
          prod_sync();
          uint32_t wp = 0;
          for (int w = 0; w < warp; ++w) wp += S.scan_ws[w];
          ++wgen;
          if ((uint32_t)tid < nb) {
            S.w_start[tid] = st0;
            S.w_pref[tid + 1] = wp + incl;
            if (bn == U.h) S.w_home = ((wgen & 0xffffffu) << 8) | (uint32_t)tid;
          }
          if (tid == 0) S.w_pref[0] = 0;
          prod_sync();
          {
            const uint32_t wh = S.w_home;
            w_hj = (wh >> 8) == (wgen & 0xffffffu) ? (int)(wh & 255u) : -1;
          }
          w_nb = nb;
          w_pos = 0;
          w_total = S.w_pref[nb];
          seg_next += nb;
          if (T.prof) pc_win += clock64() - cw0;
        }
        const long long ca0 = T.prof ? clock64() : 0;
        const uint32_t ncols = min((uint32_t)TN, w_total - w_pos);
        const bool last = (w_pos + TN >= w_total) && (seg_next >= U.s1);
        // row of candidate rank w_pos + prow: the warp finds the bin of its
        // first rank (two 32-way probes of the window prefix), then each lane
        // counts the bin boundaries among the next 32 ranks
        uint32_t q = 0xffffffffu;
        {
          const uint32_t r0 = w_pos + (prow & ~31u);
          const uint32_t step = (w_nb + 31) >> 5;
          const uint32_t c = __popc(__ballot_sync(FULL_MASK, lane * step < w_nb && S.w_pref[lane * step] <= r0));
          const uint32_t base = (c - 1) * step;  // w_pref[0] = 0 <= r0, so c >= 1
          const uint32_t b0 =
              base + __popc(__ballot_sync(FULL_MASK, (uint32_t)lane < step && base + lane < w_nb &&
                                                         S.w_pref[base + lane] <= r0)) - 1;
          const uint32_t e = b0 + 1 + lane;  // boundary after bin b0 + lane
          const uint32_t t = e <= w_nb ? S.w_pref[e] - r0 : 32u;
          const uint32_t bounds = __reduce_or_sync(FULL_MASK, t < 32u ? 1u << t : 0u);
          if (prow < ncols) {
            const uint32_t b = b0 + __popc(bounds & ((2u << lane) - 1u));
            q = S.w_start[b] + (r0 + lane - S.w_pref[b]);
          }
        }
        __nv_bfloat16 *dh, *dl;  // landing slot of the raw rows
        uint32_t* iddst;  // candidate ids
        if (RAW > 0) {
          // own-row slots, last read by this thread when it converted tile
          // issued - RAW: no wait needed
          const uint32_t rs = issued % (RAW > 0 ? RAW : 1);
          dh = Raw + rs * 2 * OPB;
          dl = dh + OPB;
          iddst = S.rid[rs];
        } else {
          const uint32_t st = issued % NS;
          const uint32_t sl = pf++ & 1;
          if (tid == 0) {
            const long long c0 = T.prof ? clock64() : 0;
            S.pflag[sl] = wait_or_abort(&S.sfree[st], ((issued / NS) & 1) ^ 1, abort_flag, T.wait_limit) ? 1u : 0u;
            if (T.prof) pw_sfree += clock64() - c0;
          }
          prod_sync();
          if (!S.pflag[sl]) return 2;
          dh = Bhi + st * OPB;
          dl = Blo + st * OPB;
          iddst = S.qid[st];
        }
        if (prow < ncols) {
          if (half == 0)
            asm volatile("cp.async.ca.shared.global [%0], [%1], 4;" ::"r"(smem_u32(&iddst[prow])), "l"(ids + q)
                         : "memory");
          load_half<KP>(dh, dl, prow, half, X + (size_t)q * P.dpad, P.dpad);
        }
        asm volatile("cp.async.commit_group;" ::: "memory");
        pq |= (ncols | (last ? 0x100u : 0u)) << (9 * (issued - tile));  // uniform queue of (columns, last)
        if (tid == 0) {
          uint32_t hcr = 0, hq = 0;
          if (w_hj >= 0) {
            const uint32_t hr0 = S.w_pref[w_hj], hr1 = S.w_pref[w_hj + 1];
            const uint32_t lo = max(hr0, w_pos) - w_pos, hi = min(hr1, w_pos + ncols) - w_pos;
            if (max(hr0, w_pos) < min(hr1, w_pos + ncols)) {
              hcr = lo | (hi << 8);
              hq = hs + (w_pos + lo - hr0);
            }
          }
          S.hx[issued & 3][0] = hcr;
          S.hx[issued & 3][1] = hq;
        }
        w_pos += TN;
        ++issued;
        if (T.prof) pc_adv += clock64() - ca0;
        return 1;
      };

      bool first = true, aborted = false;
      for (;;) {
        while (issued < tile + LA && (w_pos < w_total || seg_next < U.s1)) {
          if (advance() == 2) {
            aborted = true;
            break;
          }
        }
        if (aborted || issued == tile) break;
        const long long cc0 = T.prof ? clock64() : 0;
        switch (issued - tile - 1) {  // groups newer than this tile's
          case 0: asm volatile("cp.async.wait_group 0;" ::: "memory"); break;
          case 1: asm volatile("cp.async.wait_group 1;" ::: "memory"); break;
          default: asm volatile("cp.async.wait_group 2;" ::: "memory"); break;
        }
        if (T.prof) pc_ldw += clock64() - cc0;
        const uint32_t st = tile % NS;
        const uint32_t ncols = pq & 0xffu;
        const bool last = (pq & 0x100u) != 0u;
        pq >>= 9;
        __nv_bfloat16* bh = Bhi + st * OPB;
        __nv_bfloat16* bl = Blo + st * OPB;
        const __nv_bfloat16* sh = bh;  // raw rows: in place, or in the landing slot
        const __nv_bfloat16* sl = bl;
        if (RAW > 0) {
          const uint32_t rs = tile % (RAW > 0 ? RAW : 1);
          const uint32_t id = S.rid[rs][prow];  // own row's id (half 0 copied it)
          sh = Raw + rs * 2 * OPB;
          sl = sh + OPB;
          const uint32_t fl = pf++ & 1;
          const long long cb0 = T.prof ? clock64() : 0;
          if (tid == 0) {
            const long long c0 = T.prof ? clock64() : 0;
            S.pflag[fl] = wait_or_abort(&S.sfree[st], ((tile / NS) & 1) ^ 1, abort_flag, T.wait_limit) ? 1u : 0u;
            if (T.prof) pw_sfree += clock64() - c0;
          }
          prod_sync();
          if (T.prof) pc_bar += clock64() - cb0;
          if (!S.pflag[fl]) {
            aborted = true;
            break;
          }
          if (half == 0) S.qid[st][prow] = id;
        }
        const bool ok = prow < ncols;
        const long long cp0 = T.prof ? clock64() : 0;
        const float part = conv_pass1<KP>(sh, sl, bh, bl, prow, half, ok, S.cadd_b, -2.f, P.d, 1.f, 0.f);
        const float nq2 = row_norm(part) * 0.25f;
        float tcol = 0.f, dl = 0.f;
        if (ok && !column_threshold(tb, ra2max, nq2, &tcol, &dl)) {
          tcol = 1e30f;   // every row of this column becomes a candidate ...
          dl = INFINITY;  // ... and none is accepted without the FP64 check
        }
        const long long cp1 = T.prof ? clock64() : 0;
        if (ok && (((P.d + 1) >> 3) & 1u) == half) patch_col<KP>(bh, bl, prow, P.d + 1, nq2 - tcol);
        const long long cp2 = T.prof ? clock64() : 0;
        if (T.prof) {
          pc_p1 += cp1 - cp0;
          pc_p2 += cp2 - cp1;
        }
        if (half == 0) S.dlt[st][prow] = dl;
#pragma unroll
        for (int i = 0; i < (G + 1) / 2; ++i)
          if (2 * i + (int)half < G) S.aid[st][(2 * i + half) * TM + prow] = my_aid[i];
        if (tid == 0) {
          S.meta[st] = TileMeta{a0, na, ncols, (first ? FLAG_FIRST : 0u) | (last ? FLAG_LAST : 0u), ng,
                                S.hx[tile & 3][0], S.hx[tile & 3][1], inst};
          n_tiles += 1;
          n_cells += (unsigned long long)na * ncols;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&S.full[st]);
        if (T.prof) {
          const long long ce = clock64();
          pc_fin += ce - cp2;
          pc_conv += ce - cc0;
        }
        first = false;
        ++tile;
      }
      asm volatile("cp.async.wait_all;" ::: "memory");
      ++unit_k;
      if (aborted) {
        end_marker();
        break;
      }
    }
    if (tid == 0 && n_tiles) {
      atomicAdd(&T.ctr->tiles, n_tiles);
      atomicAdd(&T.ctr->cells, n_cells);
    }
    if (tid == 0 && T.prof) {
      atomicAdd(&T.ctr->prof[0], (unsigned long long)pw_sfree);
      atomicAdd(&T.ctr->prof[1], (unsigned long long)(clock64() - p_start));
      atomicAdd(&T.ctr->prof[7], (unsigned long long)pc_unit);
      atomicAdd(&T.ctr->prof[8], (unsigned long long)pc_win);
      atomicAdd(&T.ctr->prof[9], (unsigned long long)pc_conv);
      atomicAdd(&T.ctr->prof[14], (unsigned long long)pc_ldw);
      atomicAdd(&T.ctr->prof[16], (unsigned long long)pc_adv);
      atomicAdd(&T.ctr->prof[17], (unsigned long long)pc_bar);
      atomicAdd(&T.ctr->prof[18], (unsigned long long)pc_p1);
      atomicAdd(&T.ctr->prof[19], (unsigned long long)pc_p2);
      atomicAdd(&T.ctr->prof[20], (unsigned long long)pc_fin);
    }
    }  // two threads a row
  } else if (warp == MMA_WARP) {
    // ============================ MMA issuer
    // B tiles come in stage order; each is multiplied with the unit's ng home
    // chunks into alternating TMEM accumulators (MMA tile counter mt).
    if (lane == 0) {
      constexpr uint32_t idesc = umma_idesc(TM, TN);
      constexpr uint32_t SBO = 16u * KP;
      uint32_t tile = 0, mt = 0, unit_k = 0;
      int last_b = -1;
      uint32_t last_par = 0;
      long long mw_full = 0, mw_dfree = 0;
      const long long m_start = T.prof ? clock64() : 0;
      for (;;) {
        const uint32_t st = tile % NS;
        const long long c0 = T.prof ? clock64() : 0;
        const bool fok = wait_or_abort(&S.full[st], (tile / NS) & 1, abort_flag, T.wait_limit);
        if (T.prof) mw_full += clock64() - c0;
        if (!fok) {
          mbar_arrive(&S.dfull[mt % NACC]);
          break;
        }
        const uint32_t flags = S.meta[st].flags;
        const uint32_t ng = S.meta[st].ng;
        if (flags & FLAG_END) {
          // wake the epilogue on the next accumulator, but only once every
          // epilogue warp has taken that accumulator's previous use: an
          // arrival before that would complete a second phase of dfull[b]
          // under a warp still waiting for the first (parity aliasing)
          const uint32_t b = mt % NACC;
          wait_or_abort(&S.dfree[b], ((mt / NACC) & 1) ^ 1, abort_flag, T.wait_limit);
          mbar_arrive(&S.dfull[b]);
          break;
        }
        bool ok = true;
        if (flags & FLAG_FIRST) ok = wait_or_abort(&S.afull, unit_k & 1, abort_flag, T.wait_limit);
        if (!ok) {
          mbar_arrive(&S.dfull[mt % NACC]);
          break;
        }
        const uint32_t bh = smem_u32(Bhi + st * OPB), bl = smem_u32(Blo + st * OPB);
        for (uint32_t g = 0; g < ng && ok; ++g) {
          const uint32_t b = mt % NACC;
          const long long c1 = T.prof ? clock64() : 0;
          ok = wait_or_abort(&S.dfree[b], ((mt / NACC) & 1) ^ 1, abort_flag, T.wait_limit);
          if (T.prof) mw_dfree += clock64() - c1;
          if (!ok) {
            mbar_arrive(&S.dfull[b]);
            break;
          }
          if (T.stall_test) {  // failure-detection test: never signal, let the waits run out
            ++mt;
            continue;
          }
          asm volatile("tcgen05.fence::after_thread_sync;");
          const uint32_t ah = smem_u32(Ahi + g * OPB), al = smem_u32(Alo + g * OPB);
          const uint32_t dt = tbase + b * TN;
#pragma unroll
          for (int ks = 0; ks < KP / 16; ++ks) {
            const uint32_t o = ks * 256;
            mma_bf16(dt, umma_desc(ah + o, SBO), umma_desc(bh + o, SBO), idesc, ks > 0 ? 1u : 0u);
            mma_bf16(dt, umma_desc(ah + o, SBO), umma_desc(bl + o, SBO), idesc, 1u);
            mma_bf16(dt, umma_desc(al + o, SBO), umma_desc(bh + o, SBO), idesc, 1u);
          }
          tc_commit(&S.dfull[b]);
          last_b = (int)b;
          last_par = (mt / NACC) & 1;
          ++mt;
        }
        if (!ok) break;
        if ((flags & FLAG_LAST) && !T.stall_test) {
          tc_commit(&S.afree);
          ++unit_k;
        }
        ++tile;
      }
      if (T.prof) {
        atomicAdd(&T.ctr->prof[2], (unsigned long long)mw_full);
        atomicAdd(&T.ctr->prof[3], (unsigned long long)mw_dfree);
        atomicAdd(&T.ctr->prof[4], (unsigned long long)(clock64() - m_start));
        atomicAdd(&T.ctr->prof[12], (unsigned long long)mt);
      }
      // an aborting CTA may still have MMAs in flight: wait (bounded) for the
      // last committed tile, MMAs complete in issue order
      if (*abort_flag && last_b >= 0) {
        volatile uint32_t no_abort = 0;
        wait_or_abort(&S.dfull[last_b], last_par, &no_abort, T.wait_limit);
      }
    }
    __syncwarp();
  } else if (warp >= EPI0 && warp < EPI0 + NEPI) {
    // ============================ epilogue (NEPI warps)
    // warp w reads TMEM lane quarter w % 4 (the hardware's access rule) and
    // the 32-column blocks (w - EPI0) / 4, + NEPI / 4, ... of each 128 x 128
    // accumulator
    const uint32_t quarter = warp & 3;
    const uint32_t cblk0 = (warp - EPI0) >> 2;
    PairStage ps{pstage + (warp - EPI0) * PSTAGE, 0, 0, P.pairs_ij != 0};
    PairStage bs{pstage + (NEPI + warp - EPI0) * PSTAGE, 0};
    const RingCtx rcp_{P.pair_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
    const RingCtx rcb_{P.band_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
    const RingCtx* rcp = P.ring ? &rcp_ : nullptr;
    const RingCtx* rcb = P.ring ? &rcb_ : nullptr;
    uint32_t tile = 0, mt = 0, g = 0;
    long long ew_dfull = 0, ec_ld = 0, ec_slow = 0, ec_stage = 0;
    const long long e_start = T.prof ? clock64() : 0;
    for (;;) {
      const uint32_t st = tile % NS, b = mt % NACC;
      // all lanes wait; the outcome is made warp-uniform (tcgen05.ld is .sync.aligned)
      const long long cw = T.prof ? clock64() : 0;
      const bool ok = __all_sync(FULL_MASK, wait_or_abort(&S.dfull[b], (mt / NACC) & 1, abort_flag, T.wait_limit));
      if (T.prof) ew_dfull += clock64() - cw;
      if (!ok) break;
      const TileMeta M = S.meta[st];
      if (__any_sync(FULL_MASK, (M.flags & FLAG_END) || *abort_flag)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t row = g * TM + quarter * 32 + lane;  // row within the unit
      const bool row_ok = row < M.na;
      const uint32_t a_sorted = M.a0 + row;
#pragma unroll 1
      for (uint32_t c0 = 32 * cblk0; c0 < TN; c0 += 32 * (NEPI / 4)) {
      if (g * TM + quarter * 32 < M.na && c0 < M.ncols) {
        uint32_t v[32];
        const long long cl0 = T.prof ? clock64() : 0;
        tmem_ld32_nowait(tbase + b * TN + ((quarter * 32u) << 16) + c0, v);
        tmem_wait();
        if (T.prof) ec_ld += clock64() - cl0;
        // sign bits (D' < 0: a candidate), column c0 + j at bit j: one
        // funnel shift per value, in four independent chains of 8
        uint32_t m;
        {
          uint32_t m0 = 0, m1 = 0, m2 = 0, m3 = 0;
#pragma unroll
          for (int j = 7; j >= 0; --j) {
            m0 = __funnelshift_l(v[j], m0, 1);
            m1 = __funnelshift_l(v[8 + j], m1, 1);
            m2 = __funnelshift_l(v[16 + j], m2, 1);
            m3 = __funnelshift_l(v[24 + j], m3, 1);
          }
          m = m0 | (m1 << 8) | (m2 << 16) | (m3 << 24);
        }
        const uint32_t nvalid = min(32u, M.ncols - c0);
        if (nvalid < 32) m &= (1u << nvalid) - 1u;
        if (!row_ok) m = 0;
        uint32_t acc_bits = 0, band_bits = 0;
        const bool maybe = m != 0;
        const long long cs0 = T.prof ? clock64() : 0;
        const bool any_maybe = __any_sync(FULL_MASK, maybe);  // blocks without candidates skip the rest
        if (any_maybe) {
          if (maybe) {
            // home bin: a pair (a, q) of two home rows is kept only for a < q
            // (sorted positions); the home rows of this tile are the columns
            // [hlo, hhi), column c at position hq + c - hlo
            const uint32_t hlo = M.hcr & 255u, hhi = M.hcr >> 8;
            if (hlo < hhi && a_sorted >= M.hq) {
              const uint32_t lim = hlo + min(a_sorted - M.hq, 255u) + 1;  // columns < lim have q <= a
              const int e0 = (int)max(hlo, c0) - (int)c0, e1 = (int)min(min(hhi, lim), c0 + 32) - (int)c0;
              if (e0 < e1) m &= ~((e1 >= 32 ? FULL_MASK : ((1u << e1) - 1u)) & ~((1u << e0) - 1u));
            }
            while (m) {
              const int j = __ffs(m) - 1;
              m &= m - 1;
              if (pick32(v, j) <= -S.dlt[st][c0 + j])
                acc_bits |= 1u << j;
              else
                band_bits |= 1u << j;  // decided later in FP64 (band list)
            }
          }
        }
        __syncwarp();
        const long long cs1 = T.prof ? clock64() : 0;
        if (T.prof) ec_slow += cs1 - cs0;
        const uint32_t ia = (acc_bits | band_bits) ? S.aid[st][row] : 0u;
        auto emit = [&](PairStage& stg, uint32_t bits, unsigned long long* counter, unsigned long long* list,
                        unsigned long long lcap, unsigned long long* ip, const RingCtx* rc) {
          stage_pairs(
              stg, __popc(bits),
              [&](uint32_t) {
                const int j = __ffs(bits) - 1;
                bits &= bits - 1;
                const uint32_t iq = S.qid[st][c0 + j];
                const uint32_t lo = ia < iq ? ia : iq, hi = ia < iq ? iq : ia;
                return ((unsigned long long)lo << 32) | hi;
              },
              counter, list, lcap, ip, M.inst, rc);
        };
        if (any_maybe && __any_sync(FULL_MASK, acc_bits != 0u))
          emit(ps, acc_bits, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, rcp);
        if (any_maybe && __any_sync(FULL_MASK, band_bits != 0u))
          emit(bs, band_bits, &P.ctr->band_n, P.band_list, P.band_cap, nullptr, rcb);
        if (T.prof) ec_stage += clock64() - cs1;
      }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncwarp();
      const bool last_g = g + 1 >= M.ng;
      if (lane == 0) {
        mbar_arrive(&S.dfree[b]);
        if (last_g) mbar_arrive(&S.sfree[st]);  // the B stage served all home chunks
      }
      ++mt;
      if (last_g) {
        g = 0;
        ++tile;
      } else {
        ++g;
      }
    }
    stage_flush(ps, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, rcp);
    stage_flush(bs, &P.ctr->band_n, P.band_list, P.band_cap, nullptr, rcb);
    if (T.prof && lane == 0) {
      atomicAdd(&T.ctr->prof[5], (unsigned long long)ew_dfull);
      atomicAdd(&T.ctr->prof[6], (unsigned long long)(clock64() - e_start));
      atomicAdd(&T.ctr->prof[10], (unsigned long long)ec_ld);
      atomicAdd(&T.ctr->prof[11], (unsigned long long)ec_slow);
      atomicAdd(&T.ctr->prof[13], (unsigned long long)ec_stage);
    }
  }
  // all roles meet here before tensor memory is released
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == MMA_WARP) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 512;" ::"r"(tbase));
  if (tid == 0 && S.abort_flag) atomicExch(&P.ctr->error, 1ull);
}

// Stages and home chunks per KP within about 200 KB of operands: one CTA per
// SM (512 TMEM columns).
template <int KP>
struct TcShape {
  static constexpr int G = KP <= 32 ? 4 : (KP <= 64 ? 2 : 1);
  static constexpr int NS = KP <= 32 ? 4 : (KP <= 96 ? 3 : 2);
  // separate landing slots where they fit: four for K <= 32 (pair mode, two
  // pairs of tiles in flight), three for K = 48
  static constexpr int RAW = KP <= 32 ? 4 : (KP <= 48 ? 3 : 0);
  // short rows: many tiles, pairs and hits per converted row -> more epilogue
  // warps (16: 72 registers a thread); long rows: 8 (96 registers)
  static constexpr int NEPI = KP <= 48 ? 16 : 8;
};

template <int KP>
void launch_tc(mistic_handle_s* h, const JoinParams& P, const TcParams& T) {
  constexpr int NS = TcShape<KP>::NS, G = TcShape<KP>::G, RAW = TcShape<KP>::RAW, NEPI = TcShape<KP>::NEPI;
  constexpr int NT = tc_threads(NEPI);
  const size_t dyn = (2 * G + 2 * NS + 2 * RAW) * (size_t)TM * KP * sizeof(__nv_bfloat16) +
                     (size_t)2 * NEPI * PSTAGE * sizeof(unsigned long long);
  MCK(cudaFuncSetAttribute(k_join_tc<KP, NS, G, RAW, NEPI>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  MCK(cudaFuncSetAttribute(k_join_tc<KP, NS, G, RAW, NEPI>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int per_sm = 0;
  MCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_join_tc<KP, NS, G, RAW, NEPI>, NT, dyn));
  if (per_sm < 1) throw Error(MISTIC_ERR_TOO_LARGE, "tensor-core join does not fit on an SM");
  unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)h->sms, T.n_units);
  if (T.grid_cap) grid = std::min(grid, T.grid_cap);
  if (getenv("MISTIC_DEBUG"))
    fprintf(stderr, "[mistic] join_tc KP=%d NS=%d G=%d RAW=%d NEPI=%d dyn=%zu occupancy=%d grid=%u units=%llu\n", KP,
            NS, G, RAW, NEPI, dyn, per_sm, grid, (unsigned long long)T.n_units);
  k_join_tc<KP, NS, G, RAW, NEPI><<<grid, NT, dyn, h->stream>>>(P, T);
  launched(h, "join_tc");
}

}  // namespace

namespace join {

int tc_kp(uint32_t d) { return (int)(((d + 2) + 15) / 16 * 16); }
// Home rows per tensor-core unit: G chunks of 128 share each converted
// candidate tile (G = 2 while the operands leave room for two CTAs per SM).
// Longer rows go to the K-chunked kernel (join_tcw.cu), 256 home rows a unit.
uint32_t tc_rows(uint32_t d) {
  const int kp = tc_kp(d);
  if (kp > 128) return 256;
  return (uint32_t)TM * (kp <= 32 ? 4 : (kp <= 64 ? 2 : 1));
}
bool tc_supported(uint32_t d) { return d >= 1 && d <= MAX_D; }

void run_tc(mistic_handle_s* h, const JoinParams& P, const TcParams& T) {
  if (T.n_units == 0) return;
  switch (tc_kp(P.d)) {
    case 16: launch_tc<16>(h, P, T); break;
    case 32: launch_tc<32>(h, P, T); break;
    case 48: launch_tc<48>(h, P, T); break;
    case 64: launch_tc<64>(h, P, T); break;
    case 80: launch_tc<80>(h, P, T); break;
    case 96: launch_tc<96>(h, P, T); break;
    case 112: launch_tc<112>(h, P, T); break;
    case 128: launch_tc<128>(h, P, T); break;
    default: run_tcw(h, P, T); break;
  }
}

}  // namespace join
}  // namespace mistic
