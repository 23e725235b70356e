// Distance join over the bin index, with result-pair compaction.
//
// Reference counterpart: nodeByPoint5 + cachedDistanceCheck,
// src/kernel.cu:992-1046 and :833-865 (launched per batch at
// src/launcher.cu:3430).  There, `tpp` threads share one query point, loop
// over the neighbour nodes' points, test Σ(p - q)^2 <= ε² in FP64 and append
// every hit with a global 64-bit atomicAdd into two 2.5e9-entry arrays.
//
// Here:
//  - Work is a device list of units (a chunk of up to CH points of a home
//    bin against a segment of its neighbour-bin list, neighbours >= home),
//    drained by persistent warps through an atomic cursor, so skewed bins
//    spread over all SMs.
//  - The home chunk is staged in shared memory; each lane holds one
//    candidate row in registers and accumulates CH distances at once, so a
//    shared-memory broadcast load feeds 4 dimensions of one distance.
//  - FP32 mode filters with FP32 distances on centred coordinates and sends
//    only pairs whose FP32 value lies within a rigorous error band of ε² to
//    an FP64 re-decision with the reference predicate; FP64 mode evaluates
//    the reference predicate for every candidate.
//  - A warp votes first; only warps holding a hit or a band pair take the
//    slow path, where hits are counted with one warp scan and one atomicAdd.
#include <math.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include <type_traits>

#include "emit.cuh"
#include "internal.cuh"

namespace mistic {

constexpr int JOIN_THREADS = 256;

__device__ __forceinline__ uint32_t warp_incl_scan_u32(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// The reference predicate (src/utils.cu:296-309): sequential, each of the
// subtraction, product and sum rounded to FP64 (no contraction), on rows i
// and j of the caller's row-major array `raw` (FP32 or FP64, d columns).
__device__ __forceinline__ double exact_sqdist(const void* raw, int raw_f32, uint32_t d, uint32_t i, uint32_t j) {
  double s = 0.0;
  // loads in groups of 8 (all in flight), sums in coordinate order
  for (uint32_t t0 = 0; t0 < d; t0 += 8) {
    double av[8], bv[8];
    if (raw_f32) {
      const float* a = (const float*)raw + (size_t)i * d;
      const float* b = (const float*)raw + (size_t)j * d;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        av[k] = t0 + k < d ? (double)a[t0 + k] : 0.0;
        bv[k] = t0 + k < d ? (double)b[t0 + k] : 0.0;
      }
    } else {
      const double* a = (const double*)raw + (size_t)i * d;
      const double* b = (const double*)raw + (size_t)j * d;
#pragma unroll
      for (int k = 0; k < 8; ++k) {
        av[k] = t0 + k < d ? a[t0 + k] : 0.0;
        bv[k] = t0 + k < d ? b[t0 + k] : 0.0;
      }
    }
#pragma unroll
    for (int k = 0; k < 8; ++k) {
      if (t0 + k < d) {
        const double df = __dsub_rn(av[k], bv[k]);
        s = __dadd_rn(s, __dmul_rn(df, df));
      }
    }
  }
  return s;
}

// What a join kernel needs about the instance of one unit: the launch's own
// arrays, or in a fused batch join those of the unit's instance.
struct UnitView {
  const uint32_t* bstart;
  const uint32_t* nbr;
  const uint32_t* ids;
  const void* xs;
  float t_lo, t_hi;
  double eps2, amb;
  uint32_t inst;
};

// The pair-ring contexts of a launch (null pointers outside ring mode).
struct RingPair {
  RingCtx pairs, band;
};
__device__ __forceinline__ RingPair ring_ctx(const JoinParams& P) {
  RingPair r;
  r.pairs = RingCtx{P.pair_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
  r.band = RingCtx{P.band_tags, P.deferred, P.def_out, &P.ctr->def_n, &P.ctr->stop};
  return r;
}

// Unit of claim index t of a CUDA-core launch: first the units deferred by
// the last ring pass, then the list from main_start (the identity outside
// ring mode).  In ring mode a unit claimed after the stop is deferred unrun.
// Returns false when the worker has nothing more to do.
__device__ __forceinline__ bool claim_unit(const JoinParams& P, const RingCtx* rc, unsigned long long t,
                                           unsigned long long* u) {
  if (P.claim_cap && t >= P.claim_cap) return false;
  unsigned long long v;
  if (t < P.n_def_in) {
    v = P.def_in[t];
  } else {
    v = P.main_start + (t - P.n_def_in);
    if (v >= P.n_units) return false;
  }
  if (rc && *(volatile unsigned long long*)&P.ctr->stop) {
    ring_defer(rc, (uint32_t)v);
    return false;
  }
  *u = v;
  return true;
}

// Warp-uniform claim: lane 0 takes the next claim index.
__device__ __forceinline__ bool warp_claim(const JoinParams& P, const RingCtx* rc, unsigned long long* u) {
  unsigned long long v = ~0ull;
  if ((threadIdx.x & 31) == 0) {
    const unsigned long long t = atomicAdd(&P.ctr->next_unit, 1ull);
    if (!claim_unit(P, rc, t, &v)) v = ~0ull;
  }
  v = __shfl_sync(FULL_MASK, v, 0);
  *u = v;
  return v != ~0ull;
}

__device__ __forceinline__ UnitView unit_view(const JoinParams& P, unsigned long long u) {
  UnitView v;
  if (P.insts) {
    v.inst = P.unit_inst[u];
    const InstDesc& I = P.insts[v.inst];
    v.bstart = I.bstart;
    v.nbr = I.nbr;
    v.ids = I.ids;
    v.xs = I.xs;
    v.t_lo = I.t_lo;
    v.t_hi = I.t_hi;
    v.eps2 = I.eps2;
    v.amb = I.amb;
  } else {
    v.inst = 0;
    v.bstart = P.bstart;
    v.nbr = P.nbr;
    v.ids = P.ids;
    v.xs = P.xs;
    v.t_lo = P.t_lo;
    v.t_hi = P.t_hi;
    v.eps2 = P.eps2;
    v.amb = P.amb;
  }
  if (P.ring) v.inst = (uint32_t)u;  // the ring's tag of the unit's pairs (no fused batch in ring mode)
  return v;
}

// Stages this lane's pairs (bit a of `acc`: home point a0 + a with
// candidate q) through the warp's buffer into a pair list (accepted pairs,
// or the band list of pairs to re-decide in FP64).
__device__ __forceinline__ void stage_hits(PairStage& ps, const uint32_t* ids, uint32_t acc, uint32_t a0, uint32_t q,
                                           unsigned long long* counter, unsigned long long* list,
                                           unsigned long long cap, unsigned long long* inst_pairs, uint32_t inst,
                                           const RingCtx* rc) {
  const uint32_t iq = acc ? ids[q] : 0u;
  uint32_t bits = acc;
  stage_pairs(
      ps, __popc(acc),
      [&](uint32_t) {
        const int a = __ffs(bits) - 1;
        bits &= bits - 1;
        const uint32_t ia = ids[a0 + a];
        const uint32_t lo = ia < iq ? ia : iq, hi = ia < iq ? iq : ia;
        return ((unsigned long long)lo << 32) | hi;
      },
      counter, list, cap, inst_pairs, inst, rc);
}

__device__ __forceinline__ void add_counter(unsigned long long* c, uint32_t v) {
  const int lane = threadIdx.x & 31;
  uint32_t s = warp_incl_scan_u32(v);
  s = __shfl_sync(FULL_MASK, s, 31);
  if (lane == 0 && s) atomicAdd(c, (unsigned long long)s);
}

// Valid-home mask for candidate q: home points a0 .. a0+na-1, and when q
// lies in the home bin itself only pairs with sorted position a < q.
__device__ __forceinline__ uint32_t home_mask(uint32_t na, bool self, uint32_t q, uint32_t a0, int CH) {
  uint32_t m = na >= 32 ? FULL_MASK : ((1u << na) - 1u);
  if (self) {
    const int lim = (int)q - (int)a0;
    m &= lim >= 32 ? FULL_MASK : (lim <= 0 ? 0u : ((1u << lim) - 1u));
  }
  return CH >= 32 ? m : (m & ((1u << CH) - 1u));
}

// Candidate stream of one unit: the points of the neighbour bins
// nbr[s .. s1) in order, 32 per tile, lanes filled across bin boundaries
// (bins average a few points, so one bin per tile would leave most lanes
// idle).  `s` and `off` (next bin, offset inside it) are warp-uniform.
// Each lane gets its candidate's sorted position q, or qv = false past the
// end.  Lane l finds its bin by a binary search over the warp's inclusive
// scan of up to 32 bin sizes.
struct CandTile {
  uint32_t q;
  bool qv;
};

__device__ __forceinline__ CandTile next_tile(const uint32_t* nbr, const uint32_t* bstart, uint32_t& s, uint32_t& off,
                                              uint32_t s1) {
  const int lane = threadIdx.x & 31;
  const uint32_t bj = s + lane;
  uint32_t start = 0, size = 0;
  if (bj < s1) {
    const uint32_t b = nbr[bj];
    start = bstart[b];
    size = bstart[b + 1] - start;
    if (lane == 0) {
      start += off;
      size -= off;
    }
  }
  const uint32_t incl = warp_incl_scan_u32(size);
  const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
  // j = first window bin whose inclusive end exceeds this lane's rank
  int lo = 0, hi = 31;
#pragma unroll
  for (int it = 0; it < 5; ++it) {
    const int mid = (lo + hi) >> 1;
    const uint32_t v = __shfl_sync(FULL_MASK, incl, mid);
    if (v <= (uint32_t)lane) lo = mid + 1; else hi = mid;
  }
  const int j = lo;
  const uint32_t sj = __shfl_sync(FULL_MASK, start, j);
  const uint32_t ej = __shfl_sync(FULL_MASK, incl, j);
  const uint32_t zj = __shfl_sync(FULL_MASK, size, j);
  CandTile t;
  t.qv = (uint32_t)lane < total;
  t.q = sj + (uint32_t)lane - (ej - zj);
  // advance past the 32 candidates handed out
  if (total > 32) {
    const int j31 = __shfl_sync(FULL_MASK, j, 31);
    const uint32_t e31 = __shfl_sync(FULL_MASK, ej, 31), z31 = __shfl_sync(FULL_MASK, zj, 31);
    const uint32_t used = 32 - (e31 - z31);  // candidates taken from bin j31
    if (used < z31) {
      off = (j31 == 0 ? off : 0u) + used;
      s += j31;
    } else {
      off = 0;
      s += j31 + 1;
    }
  } else {
    s = min(s + 32, s1);
    off = 0;
  }
  return t;
}

// ---------------------------------------------------------------- FP32 filter
// Distance of lane candidate (qrow) to the CH staged home rows, dims
// [0, d): full float4 chunks, then a 1-3 wide tail; home rows beyond na are
// skipped (warp-uniform), their accumulators stay unused.
template <int CH>
__device__ __forceinline__ void f32_dists(const float4* __restrict__ qrow, const float4* sA, uint32_t nq4,
                                          uint32_t na, float (&acc)[CH]) {
  // rows are zero padded to nq4 float4 (padding adds exact zeros); packed
  // FP32 pairs as in k_join_f32r: even and odd coordinates summed apart
  unsigned long long acc2[CH];
#pragma unroll
  for (int a = 0; a < CH; ++a) acc2[a] = 0ull;
  const ulonglong2* q2 = reinterpret_cast<const ulonglong2*>(qrow);
  const ulonglong2* a2 = reinterpret_cast<const ulonglong2*>(sA);
  for (uint32_t c = 0; c < nq4; ++c) {
    const ulonglong2 qq = q2[c];
#pragma unroll
    for (int a = 0; a < CH; ++a) {
      if (a >= (int)na) break;
      const ulonglong2 aa = a2[a * nq4 + c];
      unsigned long long t;
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t) : "l"(aa.x), "l"(qq.x));
      asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(acc2[a]) : "l"(t));
      asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(t) : "l"(aa.y), "l"(qq.y));
      asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(acc2[a]) : "l"(t));
    }
  }
#pragma unroll
  for (int a = 0; a < CH; ++a) {
    float lo, hi;
    asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc2[a]));
    acc[a] = lo + hi;
  }
}

template <int CH>
__global__ void __launch_bounds__(JOIN_THREADS)
k_join_f32(const JoinParams P) {
  extern __shared__ float4 smem_f4[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nq4 = P.dpad >> 2;
  float4* sA = smem_f4 + (size_t)w * CH * nq4;
  unsigned long long* stg = reinterpret_cast<unsigned long long*>(smem_f4 + (size_t)(blockDim.x >> 5) * CH * nq4);
  PairStage ps{stg + (size_t)w * PSTAGE, 0, 0, P.pairs_ij != 0};
  PairStage bs{stg + (size_t)((blockDim.x >> 5) + w) * PSTAGE, 0};
  const RingPair RP = ring_ctx(P);
  const RingCtx* rcp = P.ring ? &RP.pairs : nullptr;
  const RingCtx* rcb = P.ring ? &RP.band : nullptr;
  for (;;) {
    unsigned long long u = 0;
    if (!warp_claim(P, rcp, &u)) break;
    const Unit U = P.units[u];
    const UnitView V = unit_view(P, u);
    const float4* X = (const float4*)V.xs;
    const uint32_t hs = V.bstart[U.h], he = V.bstart[U.h + 1];
    const uint32_t a0 = hs + U.chunk * CH;
    const uint32_t na = min((uint32_t)CH, he - a0);
    __syncwarp();
    for (uint32_t i = lane; i < CH * nq4; i += 32)
      sA[i] = i < na * nq4 ? X[(size_t)a0 * nq4 + i] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    uint32_t s = U.s0, off = 0;
    while (s < U.s1) {
      const CandTile t = next_tile(V.nbr, V.bstart, s, off, U.s1);
      const uint32_t q = t.q;
      const float4* qrow = X + (size_t)(t.qv ? q : a0) * nq4;
      float acc[CH];
      f32_dists<CH>(qrow, sA, nq4, na, acc);
      uint32_t m = 0;
#pragma unroll
      for (int a = 0; a < CH; ++a) {
        if (a >= (int)na) break;
        m |= (acc[a] <= V.t_hi ? 1u : 0u) << a;
      }
      m = t.qv ? (m & home_mask(na, q >= hs && q < he, q, a0, CH)) : 0u;
      if (__any_sync(FULL_MASK, m != 0)) {
        uint32_t lo_m = 0;
#pragma unroll
        for (int a = 0; a < CH; ++a) {
          if (a >= (int)na) break;
          lo_m |= (acc[a] <= V.t_lo ? 1u : 0u) << a;
        }
        lo_m &= m;
        const uint32_t band = m & ~lo_m;
        stage_hits(ps, V.ids, lo_m, a0, q, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, V.inst, rcp);
        if (__any_sync(FULL_MASK, band != 0u))  // decided later, all at once (k_band_check)
          stage_hits(bs, V.ids, band, a0, q, &P.ctr->band_n, P.band_list, P.band_cap, nullptr, V.inst, rcb);
      }
    }
  }
  stage_flush(ps, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, rcp);
  stage_flush(bs, &P.ctr->band_n, P.band_list, P.band_cap, nullptr, rcb);
}

// FP32 filter for d <= 32: the lane's candidate row lives in registers as DQ
// float4 chunks (compile time), the home rows are visited in groups of 8 so
// each shared-memory broadcast load feeds 8 independent FMA chains, and each
// group is classified as soon as it is complete (8 live accumulators).  HALF:
// the last chunk's second coordinate pair is padding (d <= 4 DQ - 2) and is
// skipped -- its terms are (0 - 0)^2, so the sums are unchanged (5M x 18:
// 30.6 -> 28.6 ms; groups of 2 and 6 rows for the last rows of small bins
// were measured slower, 31.9 ms).
template <int DQ, bool HALF>
__global__ void __launch_bounds__(JOIN_THREADS, (DQ <= 4 ? 4 : 3))
k_join_f32r(const JoinParams P) {
  constexpr int CH = 32;
  extern __shared__ float4 smem_f4r[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  float4* sA = smem_f4r + (size_t)w * CH * DQ;
  unsigned long long* stg = reinterpret_cast<unsigned long long*>(smem_f4r + (size_t)(blockDim.x >> 5) * CH * DQ);
  PairStage ps{stg + (size_t)w * PSTAGE, 0, 0, P.pairs_ij != 0};
  PairStage bs{stg + (size_t)((blockDim.x >> 5) + w) * PSTAGE, 0};
  const RingPair RP = ring_ctx(P);
  const RingCtx* rcp = P.ring ? &RP.pairs : nullptr;
  const RingCtx* rcb = P.ring ? &RP.band : nullptr;
  for (;;) {
    unsigned long long u = 0;
    if (!warp_claim(P, rcp, &u)) break;
    const Unit U = P.units[u];
    const UnitView V = unit_view(P, u);
    const float4* X = (const float4*)V.xs;
    const uint32_t hs = V.bstart[U.h], he = V.bstart[U.h + 1];
    const uint32_t a0 = hs + U.chunk * CH;
    const uint32_t na = min((uint32_t)CH, he - a0);
    __syncwarp();
    for (uint32_t i = lane; i < CH * DQ; i += 32)
      sA[i] = i < na * DQ ? X[(size_t)a0 * DQ + i] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncwarp();
    uint32_t s = U.s0, off = 0;
    while (s < U.s1) {
      const CandTile t = next_tile(V.nbr, V.bstart, s, off, U.s1);
      const uint32_t q = t.q;
      const ulonglong2* qrow = reinterpret_cast<const ulonglong2*>(X + (size_t)(t.qv ? q : a0) * DQ);
      ulonglong2 qq[DQ];  // the candidate row as pairs of floats
#pragma unroll
      for (int c = 0; c < DQ; ++c) qq[c] = qrow[c];
      uint32_t m = 0, lo_m = 0;
      // home rows in groups of 8 independent chains; a last group of at most
      // 4 rows (small bins: most home chunks hold a few points) takes 4.
      // Packed FP32 pairs (Blackwell f32x2, per-lane IEEE rounding): each
      // home row accumulates its even and odd coordinates separately and
      // adds the two sums at the end; the filter's error bound holds for any
      // summation order, and half the instructions are issued
      auto rows = [&](auto nr_tag, int r0) {
        constexpr int NR = decltype(nr_tag)::value;
        unsigned long long acc2[NR];
#pragma unroll
        for (int i = 0; i < NR; ++i) acc2[i] = 0ull;
#pragma unroll
        for (int c = 0; c < DQ; ++c) {
#pragma unroll
          for (int i = 0; i < NR; ++i) {
            unsigned long long tt;
            if (HALF && c == DQ - 1) {
              const unsigned long long ax = reinterpret_cast<const unsigned long long*>(sA)[2 * ((r0 + i) * DQ + c)];
              asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(tt) : "l"(ax), "l"(qq[c].x));
              asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(acc2[i]) : "l"(tt));
            } else {
              const ulonglong2 aa = reinterpret_cast<const ulonglong2*>(sA)[(r0 + i) * DQ + c];
              asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(tt) : "l"(aa.x), "l"(qq[c].x));
              asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(acc2[i]) : "l"(tt));
              asm("sub.rn.f32x2 %0, %1, %2;" : "=l"(tt) : "l"(aa.y), "l"(qq[c].y));
              asm("fma.rn.f32x2 %0, %1, %1, %0;" : "+l"(acc2[i]) : "l"(tt));
            }
          }
        }
#pragma unroll
        for (int i = 0; i < NR; ++i) {
          float lo, hi;
          asm("mov.b64 {%0, %1}, %2;" : "=f"(lo), "=f"(hi) : "l"(acc2[i]));
          const float acc = lo + hi;
          m |= (acc <= V.t_hi ? 1u : 0u) << (r0 + i);
          lo_m |= (acc <= V.t_lo ? 1u : 0u) << (r0 + i);
        }
      };
#pragma unroll
      for (int g = 0; g < CH / 8; ++g) {
        const int left = (int)na - g * 8;  // warp-uniform
        if (left <= 0) break;
        if (left <= 4)
          rows(std::integral_constant<int, 4>{}, g * 8);
        else
          rows(std::integral_constant<int, 8>{}, g * 8);
      }
      m = t.qv ? (m & home_mask(na, q >= hs && q < he, q, a0, CH)) : 0u;
      if (__any_sync(FULL_MASK, m != 0)) {
        lo_m &= m;
        const uint32_t band = m & ~lo_m;
        stage_hits(ps, V.ids, lo_m, a0, q, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, V.inst, rcp);
        if (__any_sync(FULL_MASK, band != 0u))  // decided later, all at once (k_band_check)
          stage_hits(bs, V.ids, band, a0, q, &P.ctr->band_n, P.band_list, P.band_cap, nullptr, V.inst, rcb);
      }
    }
  }
  stage_flush(ps, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, rcp);
  stage_flush(bs, &P.ctr->band_n, P.band_list, P.band_cap, nullptr, rcb);
}

// ---------------------------------------------------------------- FP64 plain
// The reference predicate for every candidate: dims in order, each
// subtraction, product and sum rounded (no contraction).
template <int CH>
__device__ __forceinline__ void f64_dists(const double2* __restrict__ qrow, const double2* sA, uint32_t nq2,
                                          uint32_t d, uint32_t na, double (&acc)[CH]) {
  const uint32_t full = d >> 1;
#pragma unroll
  for (int a = 0; a < CH; ++a) acc[a] = 0.0;
  for (uint32_t c = 0; c < full; ++c) {
    const double2 qq = qrow[c];
#pragma unroll
    for (int a = 0; a < CH; ++a) {
      if (a >= (int)na) break;
      const double2 aa = sA[a * nq2 + c];
      double t;
      t = __dsub_rn(aa.x, qq.x); acc[a] = __dadd_rn(acc[a], __dmul_rn(t, t));
      t = __dsub_rn(aa.y, qq.y); acc[a] = __dadd_rn(acc[a], __dmul_rn(t, t));
    }
  }
  if (d & 1) {
    const double2 qq = qrow[full];
#pragma unroll
    for (int a = 0; a < CH; ++a) {
      if (a >= (int)na) break;
      const double2 aa = sA[a * nq2 + full];
      const double t = __dsub_rn(aa.x, qq.x);
      acc[a] = __dadd_rn(acc[a], __dmul_rn(t, t));
    }
  }
}

template <int CH>
__global__ void __launch_bounds__(JOIN_THREADS)
k_join_f64(const JoinParams P) {
  extern __shared__ double2 smem_d2[];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const uint32_t nq2 = P.dpad >> 1;
  double2* sA = smem_d2 + (size_t)w * CH * nq2;
  PairStage ps{reinterpret_cast<unsigned long long*>(smem_d2 + (size_t)(blockDim.x >> 5) * CH * nq2) + (size_t)w * PSTAGE, 0,
               0, P.pairs_ij != 0};
  uint32_t amb_cnt = 0;
  const RingPair RP = ring_ctx(P);
  const RingCtx* rcp = P.ring ? &RP.pairs : nullptr;
  const RingCtx* rcb = P.ring ? &RP.band : nullptr;
  for (;;) {
    unsigned long long u = 0;
    if (!warp_claim(P, rcp, &u)) break;
    const Unit U = P.units[u];
    const UnitView V = unit_view(P, u);
    const double2* X = (const double2*)V.xs;
    const double thr = V.eps2 + V.amb;
    const uint32_t hs = V.bstart[U.h], he = V.bstart[U.h + 1];
    const uint32_t a0 = hs + U.chunk * CH;
    const uint32_t na = min((uint32_t)CH, he - a0);
    __syncwarp();
    for (uint32_t i = lane; i < CH * nq2; i += 32)
      sA[i] = i < na * nq2 ? X[(size_t)a0 * nq2 + i] : make_double2(0.0, 0.0);
    __syncwarp();
    uint32_t s = U.s0, off = 0;
    while (s < U.s1) {
      const CandTile t = next_tile(V.nbr, V.bstart, s, off, U.s1);
      const uint32_t q = t.q;
      const double2* qrow = X + (size_t)(t.qv ? q : a0) * nq2;
      double acc[CH];
      f64_dists<CH>(qrow, sA, nq2, P.d, na, acc);
      uint32_t m = 0;
#pragma unroll
      for (int a = 0; a < CH; ++a) {
        if (a >= (int)na) break;
        m |= (acc[a] <= thr ? 1u : 0u) << a;
      }
      m = t.qv ? (m & home_mask(na, q >= hs && q < he, q, a0, CH)) : 0u;
      if (__any_sync(FULL_MASK, m != 0)) {
        uint32_t acc_m = 0, amb_m = 0;
#pragma unroll
        for (int a = 0; a < CH; ++a) {
          acc_m |= (acc[a] <= V.eps2 ? 1u : 0u) << a;
          amb_m |= (fabs(acc[a] - V.eps2) <= V.amb ? 1u : 0u) << a;
        }
        acc_m &= m;
        amb_cnt += __popc(amb_m & m);
        stage_hits(ps, V.ids, acc_m, a0, q, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, V.inst, rcp);
      }
    }
  }
  stage_flush(ps, &P.ctr->pairs, P.pairs, P.cap, P.inst_pairs, rcp);
  add_counter(&P.ctr->ambiguous, amb_cnt);
}

// ---------------------------------------------------------------- launcher
// ---------------------------------------------------------------- band check
// The FP32 and tensor-core joins append pairs whose fast value falls inside
// the error band to P.band_list; this pass decides them with the reference
// FP64 predicate, one pair per thread, and appends the accepted ones (same
// packing) to the pair list.  The list length is read on the device.
__global__ void __launch_bounds__(256) k_band_check(const JoinParams P) {
  // ring mode: the slice [band0, band1) of the band list, entries of deferred
  // units skipped, accepted pairs written with their unit's tag (the slice
  // is sized to fit the ring); otherwise the whole list
  const unsigned long long n =
      P.ring ? P.band1 : min(*(volatile unsigned long long*)&P.ctr->band_n, P.band_cap);
  const int lane = threadIdx.x & 31;
  const unsigned long long stride = (unsigned long long)gridDim.x * blockDim.x;
  uint32_t cnt = 0, amb = 0;
  for (unsigned long long i0 = (P.ring ? P.band0 : 0) + (unsigned long long)blockIdx.x * blockDim.x +
                               (threadIdx.x & ~31u);
       i0 < n; i0 += stride) {
    const unsigned long long i = i0 + lane;
    bool acc = false;
    unsigned long long e = 0;
    uint32_t tag = 0;
    if (i < n && P.ring) {
      tag = P.band_tags[i];
      if (P.deferred[tag]) e = ~0ull;  // that unit runs again: its band entries come again
    }
    if (i < n && e != ~0ull) {
      e = P.band_list[i];
      const uint32_t gi = (uint32_t)(e >> 32), gj = (uint32_t)e;
      double sd, eps2 = P.eps2, ambv = P.amb;
      if (P.insts) {  // the pair's instance: the last one whose first global row is <= gi
        uint32_t lo = 0, hi = P.n_inst - 1;
        while (lo < hi) {
          const uint32_t mid = (lo + hi + 1) >> 1;
          if (P.inst_row0[mid] <= gi) lo = mid; else hi = mid - 1;
        }
        const InstDesc& I = P.insts[lo];
        sd = exact_sqdist(I.raw, I.raw_f32, I.d, gi - I.row0, gj - I.row0);
        eps2 = I.eps2;
        ambv = I.amb;
        if (sd <= eps2) atomicAdd(&P.inst_pairs[lo], 1ull);
      } else if (P.inv) {
        // the FP32 filter first (its bound is ~2^-24 relative where the
        // tensor cores' is ~2^-16 or wider): only its own, much narrower,
        // band goes on to the FP64 predicate
        const float4* a = reinterpret_cast<const float4*>(P.xf32 + (size_t)P.inv[gi] * P.dpad32);
        const float4* b = reinterpret_cast<const float4*>(P.xf32 + (size_t)P.inv[gj] * P.dpad32);
        float s0 = 0.f, s1 = 0.f;
        for (uint32_t c = 0; c < P.dpad32 / 4; ++c) {
          const float4 x = a[c], y = b[c];
          float t = x.x - y.x;
          s0 = fmaf(t, t, s0);
          t = x.y - y.y;
          s1 = fmaf(t, t, s1);
          t = x.z - y.z;
          s0 = fmaf(t, t, s0);
          t = x.w - y.w;
          s1 = fmaf(t, t, s1);
        }
        const float s32 = s0 + s1;
        if (s32 <= P.t_lo)
          sd = -1.0;  // accepted
        else if (s32 > P.t_hi)
          sd = INFINITY;  // rejected
        else
          sd = exact_sqdist(P.raw, P.raw_f32, P.d, gi, gj);
      } else {
        sd = exact_sqdist(P.raw, P.raw_f32, P.d, gi, gj);
      }
      ++cnt;
      if (fabs(sd - eps2) <= ambv) ++amb;
      acc = sd <= eps2;
    }
    const uint32_t m = __ballot_sync(FULL_MASK, acc);
    if (m) {
      unsigned long long base = 0;
      if (lane == 0) base = atomicAdd(&P.ctr->pairs, (unsigned long long)__popc(m));
      base = __shfl_sync(FULL_MASK, base, 0);
      if (acc && P.pairs) {
        const unsigned long long pos = base + __popc(m & ((1u << lane) - 1u));
        if (pos < P.cap) {
          P.pairs[pos] = P.pairs_ij ? pair_ij(e) : e;
          if (P.ring) P.pair_tags[pos] = tag;
        }
      }
    }
  }
  add_counter(&P.ctr->band, cnt);
  add_counter(&P.ctr->ambiguous, amb);
}

namespace join {

void run_band(mistic_handle_s* h, const JoinParams& P) {
  if (!P.band_list) return;
  k_band_check<<<(unsigned)h->sms * 8, 256, 0, h->stream>>>(P);
  launched(h, "band_check");
}

// Home points per unit for a mode and padded width: 32 (FP32) / 16 (FP64)
// while a warp's staged chunk stays within 16 KB, else 8 / 4.
int chunk_for(bool fp64, uint32_t dpad) {
  if (!fp64) return (size_t)32 * dpad * sizeof(float) <= 16 * 1024 ? 32 : 8;
  return (size_t)16 * dpad * sizeof(double) <= 16 * 1024 ? 16 : 4;
}

// Persistent launch: warps per block from the shared-memory budget (at most
// 8, at least 1), blocks = resident blocks per SM x SMs, capped by the work.
template <class K>
static void launch_persistent(mistic_handle_s* h, K kern, size_t smem_per_warp, const JoinParams& P,
                              const char* name) {
  constexpr size_t kBlockSmem = 200 * 1024;
  smem_per_warp += 2 * PSTAGE * sizeof(unsigned long long);  // pair and band staging buffers
  int warps = (int)std::min<size_t>(JOIN_THREADS / 32, std::max<size_t>(1, kBlockSmem / smem_per_warp));
  const size_t smem = smem_per_warp * warps;
  if (smem > kBlockSmem + 27 * 1024)
    throw Error(MISTIC_ERR_TOO_LARGE, "join tile does not fit in shared memory for this dimensionality");
  allow_max_dyn_smem(kern);
  int per_sm = 0;
  MCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, kern, warps * 32, smem));
  if (per_sm < 1) throw Error(MISTIC_ERR_TOO_LARGE, "join kernel does not fit on an SM for this dimensionality");
  const unsigned long long want = (P.n_units + warps - 1) / warps;
  unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)per_sm * h->sms, want ? want : 1);
  if (P.grid_cap) grid = std::min(grid, P.grid_cap);
  if (getenv("MISTIC_DEBUG"))
    fprintf(stderr, "[mistic] %s warps=%d smem=%zu occupancy=%d grid=%u units=%llu\n", name, warps, smem, per_sm, grid,
            (unsigned long long)P.n_units);
  kern<<<grid, warps * 32, smem, h->stream>>>(P);
  launched(h, name);
}

void run(mistic_handle_s* h, bool fp64, int CH, const JoinParams& P) {
  if (P.n_units == 0) return;
  if (!fp64) {
    const size_t spw = (size_t)CH * P.dpad * sizeof(float);
    if (CH == 32 && P.dpad <= 32) {
      // the last float4 chunk holds at most two coordinates: skip its padding pair
      const bool half = P.d + 2 <= P.dpad;
#define MISTIC_F32R(DQ)                                                              \
  case DQ:                                                                           \
    if (half)                                                                        \
      launch_persistent(h, k_join_f32r<DQ, true>, spw, P, "join_f32r");              \
    else                                                                             \
      launch_persistent(h, k_join_f32r<DQ, false>, spw, P, "join_f32r");             \
    return;
      switch (P.dpad / 4) {
        MISTIC_F32R(1)
        MISTIC_F32R(2)
        MISTIC_F32R(3)
        MISTIC_F32R(4)
        MISTIC_F32R(5)
        MISTIC_F32R(6)
        MISTIC_F32R(7)
        MISTIC_F32R(8)
        default: break;
      }
#undef MISTIC_F32R
    }
    if (CH == 32)
      launch_persistent(h, k_join_f32<32>, spw, P, "join_f32");
    else
      launch_persistent(h, k_join_f32<8>, spw, P, "join_f32");
  } else {
    const size_t spw = (size_t)CH * P.dpad * sizeof(double);
    if (CH == 16)
      launch_persistent(h, k_join_f64<16>, spw, P, "join_f64");
    else
      launch_persistent(h, k_join_f64<4>, spw, P, "join_f64");
  }
}

}  // namespace join
}  // namespace mistic
