// Warp-level staging of result pairs, shared by the join kernels.
//
// A warp collects accepted pairs in a small shared-memory buffer and
// reserves space in the global pair list once per flush (one atomicAdd per
// up to PSTAGE pairs, then coalesced stores), instead of one atomicAdd per
// tile that holds a hit: the pair counter is a single address that every SM
// updates, so per-tile atomics serialise in L2.  The reference appends every
// pair with its own 64-bit atomicAdd (src/kernel.cu:1040-1043).
#pragma once

#include "internal.cuh"

namespace mistic {

constexpr uint32_t PSTAGE = 64;
constexpr uint32_t RING_INVALID = 0xffffffffu;  // tag of a ring entry that holds no pair

// Streamed pair ring (mistic_opts.ring_capacity): the pair list and the band
// list have a fixed capacity and every entry carries the tag of the unit that
// wrote it.  A flush that does not fit marks its unit deferred (its entries
// are dropped when the ring is drained, and it runs again in the next pass),
// raises `stop` (no unit is claimed after it) and tags the slots it had
// reserved below the capacity as holding nothing.
struct RingCtx {
  uint32_t* tags;               // parallel to the list being written
  uint32_t* deferred;           // per unit tag: 1 once deferred in this pass
  uint32_t* def_out;            // deferred unit tags of this pass
  unsigned long long* def_n;
  unsigned long long* stop;
};

__device__ __forceinline__ void ring_defer(const RingCtx* rc, uint32_t tag) {
  if (atomicExch(&rc->deferred[tag], 1u) == 0u) rc->def_out[atomicAdd(rc->def_n, 1ull)] = tag;
  atomicExch(rc->stop, 1ull);
}

struct PairStage {
  unsigned long long* buf;  // this warp's PSTAGE slots in shared memory
  uint32_t n;               // staged pairs (warp-uniform)
  uint32_t inst = 0;        // instance of the staged pairs (fused batch joins), or unit tag (pair ring)
  bool ij = false;          // store pairs in the result's memory order (i, j) rather than packed
};

// A packed pair (i << 32 | j) in the result's memory order: i then j as two
// uint32 (little-endian), i.e. the halves swapped.
__device__ __forceinline__ unsigned long long pair_ij(unsigned long long v) { return (v >> 32) | (v << 32); }

__device__ __forceinline__ uint32_t stage_scan(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// Warp-collective: moves the staged pairs to the global list.  inst_pairs
// (fused batch joins, accepted-pair list only): per-instance pair counts.
__device__ __forceinline__ void stage_flush(PairStage& ps, unsigned long long* counter,
                                            unsigned long long* pairs, unsigned long long cap,
                                            unsigned long long* inst_pairs = nullptr, const RingCtx* rc = nullptr) {
  if (ps.n == 0) return;
  const int lane = threadIdx.x & 31;
  unsigned long long base = 0;
  if (lane == 0) {
    base = atomicAdd(counter, (unsigned long long)ps.n);
    if (inst_pairs) atomicAdd(&inst_pairs[ps.inst], (unsigned long long)ps.n);
  }
  base = __shfl_sync(FULL_MASK, base, 0);
  if (rc) {
    const bool fits = base + ps.n <= cap;
    for (uint32_t i = lane; i < ps.n; i += 32) {
      const unsigned long long pos = base + i;
      if (pos < cap) {
        if (fits) pairs[pos] = ps.buf[i];
        rc->tags[pos] = fits ? ps.inst : RING_INVALID;
      }
    }
    if (!fits && lane == 0) ring_defer(rc, ps.inst);
  } else if (pairs) {
    for (uint32_t i = lane; i < ps.n; i += 32) {
      const unsigned long long pos = base + i;
      if (pos < cap) pairs[pos] = ps.buf[i];
    }
  }
  __syncwarp();
  ps.n = 0;
}

// Warp-collective: adds this lane's `cnt` pairs, produced in order by
// `pair_of(k)` for k = 0..cnt-1 (packed (i << 32 | j), i < j), of instance
// `inst` (warp-uniform; 0 outside fused batch joins).
template <class F>
__device__ __forceinline__ void stage_pairs(PairStage& ps, uint32_t cnt, F pair_of, unsigned long long* counter,
                                            unsigned long long* pairs, unsigned long long cap,
                                            unsigned long long* inst_pairs = nullptr, uint32_t inst = 0,
                                            const RingCtx* rc = nullptr) {
  uint32_t incl, total;
  if (__ballot_sync(FULL_MASK, cnt > 1) == 0) {  // at most one pair per lane: prefix by ballot
    const uint32_t m1 = __ballot_sync(FULL_MASK, cnt != 0);
    incl = __popc(m1 & (0xffffffffu >> (31 - (threadIdx.x & 31))));
    total = __popc(m1);
  } else {
    incl = stage_scan(cnt);
    total = __shfl_sync(FULL_MASK, incl, 31);
  }
  if (total == 0) return;
  if (ps.n + total > PSTAGE || (ps.n && ps.inst != inst)) stage_flush(ps, counter, pairs, cap, inst_pairs, rc);
  ps.inst = inst;
  if (total > PSTAGE) {  // a dense block: reserve directly
    const int lane = threadIdx.x & 31;
    unsigned long long base = 0;
    if (lane == 31) {
      base = atomicAdd(counter, (unsigned long long)total);
      if (inst_pairs) atomicAdd(&inst_pairs[inst], (unsigned long long)total);
    }
    base = __shfl_sync(FULL_MASK, base, 31);
    const bool fits = !rc || base + total <= cap;
    if (pairs) {
      unsigned long long pos = base + incl - cnt;
      for (uint32_t k = 0; k < cnt; ++k, ++pos)
        if (pos < cap) {
          if (fits) pairs[pos] = ps.ij ? pair_ij(pair_of(k)) : pair_of(k);
          if (rc) rc->tags[pos] = fits ? inst : RING_INVALID;
        }
    }
    if (!fits && lane == 31) ring_defer(rc, inst);
    return;
  }
  if (pairs) {
    uint32_t pos = ps.n + incl - cnt;
    for (uint32_t k = 0; k < cnt; ++k) ps.buf[pos + k] = ps.ij ? pair_ij(pair_of(k)) : pair_of(k);
  }
  __syncwarp();
  ps.n += total;
}

}  // namespace mistic
