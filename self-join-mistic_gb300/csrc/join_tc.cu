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
//   - bf16 splitting: each product carries <= 3.02 * 2^-18 |A_k||B_k|,
//   - tensor-core FP32 accumulation: taken as <= 2^-19 per MMA instruction
//     relative to the sum of |products| (a generous allowance),
//   - FP32 norms (g_d), the FP32 centring (2uR + u(|a'|+|q'|)),
// with sum_k |A_k||B_k| <= (|a'| + |q'|)^2.  Rows whose bound exceeds
// 0.1 eps2 are re-decided entirely in FP64 (T_lo = -1, T_hi = inf).
//
// Data movement: operands are converted from the sorted FP32 rows by the
// CTA's threads straight into the no-swizzle K-major core-matrix layout
// (8 rows x 16 bytes per core matrix; LBO = 128 B between K-adjacent core
// matrices, SBO = 16*KP B between 8-row groups), then one elected thread
// issues the MMAs and commits to an mbarrier; all 8 warps read the 128 x 128
// FP32 tile back with tcgen05.ld (warp w: TMEM lanes 32*(w%4).., columns
// 64*(w/4)..).  Every mbarrier wait is bounded; on expiry the CTA records
// an error, stops, and releases its tensor memory.
#include <cuda_bf16.h>
#include <math.h>

#include <algorithm>
#include <cstdio>
#include <cstdlib>

#include "emit.cuh"
#include "internal.cuh"

namespace mistic {
namespace {

constexpr int TM = 128;          // home rows per tile (MMA M)
constexpr int TN = 128;          // candidate columns per tile (MMA N)
constexpr int WIN = 256;         // neighbour bins per candidate window
constexpr long long kWaitLimit = 1ll << 22;
constexpr int SV_STRIDE = 36;    // per-lane scratch row (floats), 16-B aligned

__device__ __forceinline__ uint32_t smem_u32(const void* p) { return (uint32_t)__cvta_generic_to_shared(p); }

// tcgen05 shared-memory matrix descriptor: no swizzle, K-major.
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t sbo) {
  uint64_t d = 0;
  d |= (uint64_t)((saddr >> 4) & 0x3FFF);
  d |= (uint64_t)((128u >> 4) & 0x3FFF) << 16;  // LBO: next core matrix along K
  d |= (uint64_t)((sbo >> 4) & 0x3FFF) << 32;   // SBO: next 8-row group
  d |= (uint64_t)1 << 46;                        // descriptor version
  return d;
}

// Instruction descriptor, kind::f16: D f32, A/B bf16, both K-major, N x M.
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

// Issues one 32-column TMEM load without waiting (pair with tmem_wait).
__device__ __forceinline__ void tmem_ld32_nowait(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
}
__device__ __forceinline__ void tmem_wait() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }


__device__ __forceinline__ double exact_sqdist_tc(const JoinParams& P, uint32_t i, uint32_t j) {
  double s = 0.0;
  if (P.raw_f32) {
    const float* a = (const float*)P.raw + (size_t)i * P.d;
    const float* b = (const float*)P.raw + (size_t)j * P.d;
    for (uint32_t t = 0; t < P.d; ++t) {
      const double df = __dsub_rn((double)a[t], (double)b[t]);
      s = __dadd_rn(s, __dmul_rn(df, df));
    }
  } else {
    const double* a = (const double*)P.raw + (size_t)i * P.d;
    const double* b = (const double*)P.raw + (size_t)j * P.d;
    for (uint32_t t = 0; t < P.d; ++t) {
      const double df = __dsub_rn(a[t], b[t]);
      s = __dadd_rn(s, __dmul_rn(df, df));
    }
  }
  return s;
}

__device__ __forceinline__ uint32_t warp_scan_incl(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

// ---------------------------------------------------------------- pipeline
// One CTA = 9 warps:
//   warps 0-3  producers: fetch units, convert the unit's home rows (A, once
//              per unit) and each tile's 128 candidate rows (B) into a ring of
//              NS shared-memory stages, with the per-column threshold folded
//              into B (column d+1 holds |q'|^2 - T(n));
//   warp 8     MMA issuer (one lane): 3 * KP/16 tcgen05.mma per tile into one
//              of two TMEM accumulators, tcgen05.commit to signal completion;
//   warps 4-7  epilogue: tcgen05.ld of TMEM lanes 32*(w-4).., sign-bit test
//              (D' < 0 marks a candidate), exact decision, pair emission.
// Barriers (all waits bounded):
//   full[s]   producers -> MMA        (128 arrivals)
//   sfree[s]  epilogue  -> producers  (4 arrivals; stage s and its metadata reusable)
//   dfull[b]  MMA       -> epilogue   (tcgen05.commit, or a plain arrive on the terminate tile)
//   dfree[b]  epilogue  -> MMA        (4 arrivals; accumulator b reusable)
//   afull     producers -> MMA        (128 arrivals per unit: A written)
//   afree     MMA       -> producers  (tcgen05.commit after a unit's last tile)
constexpr int TC_WARPS = 9;
constexpr int TC_THREADS2 = TC_WARPS * 32;
constexpr int NPROD = 128;
constexpr uint32_t FLAG_FIRST = 1, FLAG_LAST = 2, FLAG_END = 4;

struct TileMeta {
  uint32_t a0, na, hs, he, ncols, flags, ng;  // ng: 128-row MMA tiles of this unit (1..G)
};

template <int NS, int G>
struct TcShared2 {
  __align__(16) float center[128];
  uint32_t qpos[NS][TN];
  uint32_t qid[NS][TN];      // original row ids of the candidates
  uint32_t aid[NS][TM * G];  // original row ids of the home rows (per stage: the epilogue
                             // may still read a finished unit while producers start the next)
  float dlt[NS][TN];  // accept when D' <= -dlt
  TileMeta meta[NS];
  uint32_t w_start[WIN];
  uint32_t w_pref[WIN + 1];
  uint32_t scan_ws[4];
  unsigned long long unit;
  uint32_t w_total, w_pos, seg_next, w_nb;
  uint32_t ra2max;  // float bits, non-negative
  uint32_t abort_flag;
  uint32_t tmem_base;
  uint32_t pflag;  // producer-wide decision, written by producer thread 0
  unsigned long long full[NS], sfree[NS], dfull[2], dfree[2], afull, afree;
};

__device__ __forceinline__ void mbar_init(unsigned long long* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_u32(b)) : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
               : "memory");
}
__device__ __forceinline__ void prod_sync() { asm volatile("bar.sync 1, 128;" ::: "memory"); }

// Bounded wait; on expiry raise the CTA's abort flag.  Returns false if the
// CTA is aborting (now or already).
__device__ __forceinline__ bool wait_or_abort(unsigned long long* b, uint32_t parity, volatile uint32_t* abort_flag,
                                              long long limit = kWaitLimit) {
  const uint32_t a = smem_u32(b);
  for (long long it = 0; it < limit; ++it) {
    uint32_t done;
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(a), "r"(parity));
    if (done) return true;
    if ((it & 255) == 255 && *abort_flag) return false;
  }
  *abort_flag = 1u;
  return false;
}

// One augmented operand row, hi and lo parts.  k < d: scale * (x[k] - c[k]);
// A rows (is_a): [.., |a'|^2, 1]; B rows: [.., 1, |q'|^2 - tcol].
// FP32 norm of the centred row, sum over k < d of (x[k] - c[k])^2.  The
// row is read in groups of 8 float4 with all loads of a group in flight.
__device__ __forceinline__ float row_norm(const float* __restrict__ x, const float* c, uint32_t d, uint32_t dpad) {
  float nrm = 0.f;
  for (uint32_t g = 0; g < dpad; g += 32) {
    float4 xv[8];
#pragma unroll
    for (int i = 0; i < 8; ++i)
      xv[i] = g + 4 * i < dpad ? *reinterpret_cast<const float4*>(x + g + 4 * i) : make_float4(0.f, 0.f, 0.f, 0.f);
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const uint32_t k = g + 4 * i;
      const float4 cv = k < dpad ? *reinterpret_cast<const float4*>(c + k) : make_float4(0.f, 0.f, 0.f, 0.f);
      const float xs[4] = {xv[i].x, xv[i].y, xv[i].z, xv[i].w}, cs[4] = {cv.x, cv.y, cv.z, cv.w};
#pragma unroll
      for (int j = 0; j < 4; ++j) {
        if (k + j < d) {
          const float t = xs[j] - cs[j];
          nrm = fmaf(t, t, nrm);
        }
      }
    }
  }
  return nrm;
}

template <int KP>
__device__ __forceinline__ void write_row2(__nv_bfloat16* hi_base, __nv_bfloat16* lo_base, uint32_t r,
                                           const float* __restrict__ x, const float* c, uint32_t d, uint32_t dpad,
                                           bool is_a, float nrm, float tcol_in) {
  const float tcol = is_a ? 0.f : tcol_in;
  const float ed = is_a ? nrm : 1.f;
  const float ed1 = is_a ? 1.f : nrm - tcol;
  const float scale = is_a ? 1.f : -2.f;
#pragma unroll
  for (int kb = 0; kb < KP / 8; ++kb) {
    float v[8];
#pragma unroll
    for (int h = 0; h < 2; ++h) {
      const uint32_t k4 = kb * 8 + h * 4;
      float4 xv = make_float4(0.f, 0.f, 0.f, 0.f);
      if (k4 < dpad) xv = *reinterpret_cast<const float4*>(x + k4);
      const float xs[4] = {xv.x, xv.y, xv.z, xv.w};
#pragma unroll
      for (int i = 0; i < 4; ++i) {
        const uint32_t k = k4 + i;
        float t = 0.f;
        if (k < d) t = (xs[i] - c[k]) * scale;
        if (k == d) t = ed;
        if (k == d + 1) t = ed1;
        v[h * 4 + i] = t;
      }
    }
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
    const uint32_t off = (((r >> 3) * (KP / 8) + kb) * 64) + (r & 7) * 8;
    *reinterpret_cast<uint4*>(hi_base + off) = oh;
    *reinterpret_cast<uint4*>(lo_base + off) = ol;
  }
}

template <int KP>
__device__ __forceinline__ void zero_row2(__nv_bfloat16* hi_base, __nv_bfloat16* lo_base, uint32_t r) {
  const uint4 z = make_uint4(0, 0, 0, 0);
#pragma unroll
  for (int kb = 0; kb < KP / 8; ++kb) {
    const uint32_t off = (((r >> 3) * (KP / 8) + kb) * 64) + (r & 7) * 8;
    *reinterpret_cast<uint4*>(hi_base + off) = z;
    *reinterpret_cast<uint4*>(lo_base + off) = z;
  }
}

// Per-column threshold T(n) folded into B and the accept distance dlt(n),
// from the unit's largest |a'|^2 and this column's |q'|^2 (FP32, rounded
// outward).  Returns false when the bound is too wide to decide anything
// (the column is then re-decided entirely in FP64).
__device__ __forceinline__ bool column_threshold(const TcParams& T, float ra2max, float nq2, float* tcol,
                                                 float* dlt) {
  const float ra = sqrtf(ra2max * T.ginf), rq = sqrtf(nq2 * T.ginf);
  const float rs = ra + rq;
  const float delta = T.uR2 + T.u1 * rs;
  const float E = (T.kappa * (rs * rs + 1.2f * T.eps2_hi) + delta * (2.f * T.Dp + delta)) * 1.001f;
  if (!(E <= T.cap)) return false;
  float t = T.eps2_hi + E + T.margin;
  t += fabsf(t) * 1e-6f;
  float dl = (T.eps2_hi - T.eps2_lo) + 2.f * E + T.margin;
  dl += fabsf(dl) * 1e-6f;
  *tcol = t;
  *dlt = dl;
  return true;
}

template <int KP, int NS, int G>
__global__ void __launch_bounds__(TC_THREADS2, 2) k_join_tc(const JoinParams P, const TcParams T) {
  extern __shared__ __align__(128) unsigned char tc_dyn[];
  __shared__ TcShared2<NS, G> S;
  constexpr uint32_t OPB = TM * KP;  // bf16 elements per operand buffer
  __nv_bfloat16* Ahi = reinterpret_cast<__nv_bfloat16*>(tc_dyn);  // G home chunks of 128 rows
  __nv_bfloat16* Alo = Ahi + G * OPB;
  __nv_bfloat16* Bhi = Alo + G * OPB;  // NS stages of hi, then NS stages of lo
  __nv_bfloat16* Blo = Bhi + NS * OPB;
  float* sv = reinterpret_cast<float*>(Blo + NS * OPB);  // 4 epilogue warps x 32 lanes x SV_STRIDE
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* X = (const float*)P.xs;
  volatile uint32_t* abort_flag = &S.abort_flag;

  if (tid == 0) {
    for (int i = 0; i < NS; ++i) {
      mbar_init(&S.full[i], NPROD);
      mbar_init(&S.sfree[i], 4);
    }
    for (int i = 0; i < 2; ++i) {
      mbar_init(&S.dfull[i], 1);
      mbar_init(&S.dfree[i], 4);
    }
    mbar_init(&S.afull, NPROD);
    mbar_init(&S.afree, 1);
    asm volatile("fence.mbarrier_init.release.cluster;");
    S.abort_flag = 0;
  }
  if (warp == 8) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 256;" ::"r"(smem_u32(&S.tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = S.tmem_base;

  if (warp < 4) {
    // ============================ producers
    // Every branch that leads to bar.sync is taken on a value all 128
    // producer threads read from shared memory after the same bar.sync, so
    // the 4 warps never diverge around it; barrier waits are done by thread 0
    // and broadcast through S.pflag.
    uint32_t tile = 0, unit_k = 0;
    unsigned long long n_tiles = 0, n_cells = 0;
    long long pw_sfree = 0;
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
      if (tid == 0) {
        const unsigned long long uu = atomicAdd(&T.ctr->next_unit, 1ull);
        S.unit = uu;
        bool go = uu < T.n_units && !*abort_flag;
        if (go && unit_k > 0) go = wait_or_abort(&S.afree, (unit_k - 1) & 1, abort_flag, T.wait_limit);  // A no longer read
        S.pflag = go ? 1u : 0u;
      }
      prod_sync();
      if (!S.pflag) {
        end_marker();
        break;
      }
      const unsigned long long u = S.unit;
      const Unit U = T.units[u];
      const uint32_t hs = P.bstart[U.h], he = P.bstart[U.h + 1];
      const uint32_t a0 = hs + U.chunk * (TM * G);
      const uint32_t na = min((uint32_t)(TM * G), he - a0);
      const uint32_t ng = (na + TM - 1) / TM;
      if (tid < (int)P.dpad) S.center[tid] = X[(size_t)a0 * P.dpad + tid];
      if (tid == 0) S.ra2max = 0;
      prod_sync();
      uint32_t my_aid[G];  // original ids of home rows tid, 128 + tid, ...
#pragma unroll
      for (int g = 0; g < G; ++g) my_aid[g] = (uint32_t)(g * TM + tid) < na ? P.ids[a0 + g * TM + tid] : 0u;
      {
        float m = 0.f;
        for (uint32_t g = 0; g < ng; ++g) {
          const uint32_t r = g * TM + tid;
          if (r < na) {
            const float* xr = X + (size_t)(a0 + r) * P.dpad;
            const float nrm = row_norm(xr, S.center, P.d, P.dpad);
            write_row2<KP>(Ahi + g * OPB, Alo + g * OPB, tid, xr, S.center, P.d, P.dpad, true, nrm, 0.f);
            m = fmaxf(m, nrm);
          } else {
            zero_row2<KP>(Ahi + g * OPB, Alo + g * OPB, tid);
          }
        }
#pragma unroll
        for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL_MASK, m, o));
        if (lane == 0) atomicMax(&S.ra2max, __float_as_uint(m));
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
      mbar_arrive(&S.afull);
      if (tid == 0) {
        S.seg_next = U.s0;
        S.w_total = 0;
        S.w_pos = 0;
      }
      prod_sync();
      const float ra2max = __uint_as_float(S.ra2max);
      bool first = true, aborted = false;
      for (;;) {
        if (S.w_pos >= S.w_total) {
          const uint32_t sn = S.seg_next;
          if (sn >= U.s1) break;
          const uint32_t nb = min((uint32_t)WIN, U.s1 - sn);
          // 128 producer threads load up to 256 bins: two per thread
          uint32_t st0 = 0, sz0 = 0, st1 = 0, sz1 = 0;
          const uint32_t j0 = 2 * tid, j1 = 2 * tid + 1;
          if (j0 < nb) {
            const uint32_t b = P.nbr[sn + j0];
            st0 = P.bstart[b];
            sz0 = P.bstart[b + 1] - st0;
          }
          if (j1 < nb) {
            const uint32_t b = P.nbr[sn + j1];
            st1 = P.bstart[b];
            sz1 = P.bstart[b + 1] - st1;
          }
          const uint32_t pair = sz0 + sz1;
          const uint32_t incl = warp_scan_incl(pair);
          if (lane == 31) S.scan_ws[warp] = incl;
          prod_sync();
          uint32_t wp = 0;
          for (int w = 0; w < warp; ++w) wp += S.scan_ws[w];
          const uint32_t ex = wp + incl - pair;
          if (j0 < nb) {
            S.w_start[j0] = st0;
            S.w_pref[j0 + 1] = ex + sz0;
          }
          if (j1 < nb) {
            S.w_start[j1] = st1;
            S.w_pref[j1 + 1] = ex + sz0 + sz1;
          }
          if (tid == 0) {
            S.w_pref[0] = 0;
            S.w_nb = nb;
            S.w_pos = 0;
            S.seg_next = sn + nb;
          }
          prod_sync();
          if (tid == 0) S.w_total = S.w_pref[nb];
          prod_sync();
          continue;
        }
        const uint32_t st = tile % NS;
        if (tid == 0) {
          const long long c0 = T.prof ? clock64() : 0;
          S.pflag = wait_or_abort(&S.sfree[st], ((tile / NS) & 1) ^ 1, abort_flag, T.wait_limit) ? 1u : 0u;
          if (T.prof) pw_sfree += clock64() - c0;
        }
        prod_sync();
        if (!S.pflag) {
          aborted = true;
          break;
        }
        const uint32_t wpos = S.w_pos, wtot = S.w_total;
        const uint32_t ncols = min((uint32_t)TN, wtot - wpos);
        const bool last = (wpos + TN >= wtot) && (S.seg_next >= U.s1);
        // candidate position of column tid
        uint32_t q = 0xffffffffu;
        if ((uint32_t)tid < ncols) {
          const uint32_t rank = wpos + tid;
          int lo = 0, hi = (int)S.w_nb - 1;
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S.w_pref[mid] <= rank) lo = mid; else hi = mid - 1;
          }
          q = S.w_start[lo] + (rank - S.w_pref[lo]);
        }
        S.qpos[st][tid] = q;
        S.qid[st][tid] = (uint32_t)tid < ncols ? P.ids[q] : 0u;
#pragma unroll
        for (int g = 0; g < G; ++g) S.aid[st][g * TM + tid] = my_aid[g];
        __nv_bfloat16* bh = Bhi + st * OPB;
        __nv_bfloat16* bl = Blo + st * OPB;
        if ((uint32_t)tid < ncols) {
          const float* xr = X + (size_t)q * P.dpad;
          // norm first (the threshold depends on it), then the row
          const float nq2 = row_norm(xr, S.center, P.d, P.dpad);
          float tcol, dl;
          if (!column_threshold(T, ra2max, nq2, &tcol, &dl)) {
            tcol = 1e30f;    // every row of this column becomes a candidate ...
            dl = INFINITY;   // ... and none is accepted without the FP64 check
          }
          write_row2<KP>(bh, bl, tid, xr, S.center, P.d, P.dpad, false, nq2, tcol);
          S.dlt[st][tid] = dl;
        } else {
          zero_row2<KP>(bh, bl, tid);
          S.dlt[st][tid] = 0.f;
        }
        if (tid == 0) {
          S.meta[st] = TileMeta{a0, na, hs, he, ncols, (first ? FLAG_FIRST : 0u) | (last ? FLAG_LAST : 0u), ng};
          n_tiles += 1;
          n_cells += (unsigned long long)na * ncols;
        }
        asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
        mbar_arrive(&S.full[st]);
        first = false;
        ++tile;
        prod_sync();
        if (tid == 0) S.w_pos = wpos + TN;
        prod_sync();
      }
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
    }
  } else if (warp == 8) {
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
          mbar_arrive(&S.dfull[mt & 1]);
          break;
        }
        const uint32_t flags = S.meta[st].flags;
        const uint32_t ng = S.meta[st].ng;
        if (flags & FLAG_END) {
          mbar_arrive(&S.dfull[mt & 1]);
          break;
        }
        bool ok = true;
        if (flags & FLAG_FIRST) ok = wait_or_abort(&S.afull, unit_k & 1, abort_flag, T.wait_limit);
        if (!ok) {
          mbar_arrive(&S.dfull[mt & 1]);
          break;
        }
        const uint32_t bh = smem_u32(Bhi + st * OPB), bl = smem_u32(Blo + st * OPB);
        for (uint32_t g = 0; g < ng && ok; ++g) {
          const uint32_t b = mt & 1;
          const long long c1 = T.prof ? clock64() : 0;
          ok = wait_or_abort(&S.dfree[b], ((mt >> 1) & 1) ^ 1, abort_flag, T.wait_limit);
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
          last_par = (mt >> 1) & 1;
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
      }
      // an aborting CTA may still have MMAs in flight: wait (bounded) for the
      // last committed tile, MMAs complete in issue order
      if (*abort_flag && last_b >= 0) {
        volatile uint32_t no_abort = 0;
        wait_or_abort(&S.dfull[last_b], last_par, &no_abort, T.wait_limit);
      }
    }
    __syncwarp();
  } else {
    // ============================ epilogue (warps 4-7)
    const uint32_t quarter = warp - 4;
    float* my_sv = sv + (size_t)(quarter * 32 + lane) * SV_STRIDE;
    PairStage ps{reinterpret_cast<unsigned long long*>(sv + (size_t)4 * 32 * SV_STRIDE) + quarter * PSTAGE, 0};
    uint32_t band_cnt = 0, amb_cnt = 0;
    uint32_t tile = 0, mt = 0, g = 0;
    long long ew_dfull = 0;
    const long long e_start = T.prof ? clock64() : 0;
    for (;;) {
      const uint32_t st = tile % NS, b = mt & 1;
      // all lanes wait; the outcome is made warp-uniform (tcgen05.ld is .sync.aligned)
      const long long c0 = T.prof ? clock64() : 0;
      const bool ok = __all_sync(FULL_MASK, wait_or_abort(&S.dfull[b], (mt >> 1) & 1, abort_flag, T.wait_limit));
      if (T.prof) ew_dfull += clock64() - c0;
      if (!ok) break;
      const TileMeta M = S.meta[st];
      if (__any_sync(FULL_MASK, (M.flags & FLAG_END) || *abort_flag)) break;
      asm volatile("tcgen05.fence::after_thread_sync;");
      const uint32_t row = g * TM + quarter * 32 + lane;  // row within the unit
      const bool row_ok = row < M.na;
      const uint32_t a_sorted = M.a0 + row;
      // a quarter whose 32 rows all lie past the home chunk has nothing to do;
      // TMEM is read two 32-column chunks at a time (both loads in flight)
      auto process_chunk = [&](const uint32_t (&v)[32], uint32_t c0) {
        uint32_t o = 0;
#pragma unroll
        for (int j = 0; j < 32; ++j) o |= v[j];
        uint32_t acc_bits = 0;
        const uint32_t nvalid = M.ncols > c0 ? min(32u, M.ncols - c0) : 0u;
        const bool maybe = row_ok && nvalid && (o >> 31);
        if (__any_sync(FULL_MASK, maybe)) {
          if (maybe) {
            uint32_t m = 0;
#pragma unroll
            for (int j = 0; j < 32; ++j) m |= (v[j] >> 31) << j;
            m &= nvalid >= 32 ? FULL_MASK : ((1u << nvalid) - 1u);
#pragma unroll
            for (int j = 0; j < 32; j += 4)
              *reinterpret_cast<float4*>(my_sv + j) =
                  make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]), __uint_as_float(v[j + 2]),
                              __uint_as_float(v[j + 3]));
            while (m) {
              const int j = __ffs(m) - 1;
              m &= m - 1;
              const uint32_t q = S.qpos[st][c0 + j];
              if (q >= M.hs && q < M.he && q <= a_sorted) continue;  // home bin: only a < q
              if (my_sv[j] <= -S.dlt[st][c0 + j]) {
                acc_bits |= 1u << j;
              } else {
                const double sd = exact_sqdist_tc(P, S.aid[st][row], S.qid[st][c0 + j]);
                ++band_cnt;
                if (fabs(sd - P.eps2) <= P.amb) ++amb_cnt;
                if (sd <= P.eps2) acc_bits |= 1u << j;
              }
            }
          }
        }
        {
          const uint32_t ia = acc_bits ? S.aid[st][row] : 0u;
          uint32_t bits = acc_bits;
          stage_pairs(
              ps, __popc(acc_bits),
              [&](uint32_t) {
                const int j = __ffs(bits) - 1;
                bits &= bits - 1;
                const uint32_t iq = S.qid[st][c0 + j];
                const uint32_t lo = ia < iq ? ia : iq, hi = ia < iq ? iq : ia;
                return ((unsigned long long)lo << 32) | hi;
              },
              &P.ctr->pairs, P.pairs, P.cap);
        }
            };
      if (g * TM + quarter * 32 < M.na) {
        for (uint32_t c0 = 0; c0 < M.ncols; c0 += 64) {
          uint32_t v0[32], v1[32];
          const uint32_t ta = tbase + b * TN + ((quarter * 32u) << 16) + c0;
          tmem_ld32_nowait(ta, v0);
          tmem_ld32_nowait(ta + 32, v1);
          tmem_wait();
          process_chunk(v0, c0);
          if (c0 + 32 < M.ncols) process_chunk(v1, c0 + 32);
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
    stage_flush(ps, &P.ctr->pairs, P.pairs, P.cap);
    if (T.prof && lane == 0) {
      atomicAdd(&T.ctr->prof[5], (unsigned long long)ew_dfull);
      atomicAdd(&T.ctr->prof[6], (unsigned long long)(clock64() - e_start));
    }
    const uint32_t bt = __shfl_sync(FULL_MASK, warp_scan_incl(band_cnt), 31);
    const uint32_t at = __shfl_sync(FULL_MASK, warp_scan_incl(amb_cnt), 31);
    if (lane == 0) {
      if (bt) atomicAdd(&P.ctr->band, (unsigned long long)bt);
      if (at) atomicAdd(&P.ctr->ambiguous, (unsigned long long)at);
    }
  }
  // all roles meet here before tensor memory is released
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 8) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 256;" ::"r"(tbase));
  if (tid == 0 && S.abort_flag) atomicExch(&P.ctr->error, 1ull);
}

template <int KP>
void launch_tc(mistic_handle_s* h, const JoinParams& P, const TcParams& T) {
  constexpr int NS = KP <= 64 ? 3 : 2;
  constexpr int G = KP <= 32 ? 2 : 1;  // home chunks per unit (must match tc_rows)
  const size_t dyn = (2 * G + 2 * NS) * (size_t)TM * KP * sizeof(__nv_bfloat16) +
                     (size_t)4 * 32 * SV_STRIDE * sizeof(float) + 4 * PSTAGE * sizeof(unsigned long long);
  MCK(cudaFuncSetAttribute(k_join_tc<KP, NS, G>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  MCK(cudaFuncSetAttribute(k_join_tc<KP, NS, G>, cudaFuncAttributePreferredSharedMemoryCarveout, 100));
  int per_sm = 0;
  MCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_join_tc<KP, NS, G>, TC_THREADS2, dyn));
  if (per_sm < 1) throw Error(MISTIC_ERR_TOO_LARGE, "tensor-core join does not fit on an SM");
  const int occ = per_sm;
  // two CTAs per SM: 256 TMEM columns each (512 per SM), and registers and
  // shared memory allow two for every KP <= 64; the occupancy query reports
  // one for this 9-warp block, so it only serves as the fits-at-all check
  per_sm = (dyn + sizeof(TcShared2<NS, G>) + 1024) * 2 <= 228 * 1024 ? 2 : 1;
  const unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)per_sm * h->sms, T.n_units);
  if (getenv("MISTIC_DEBUG"))
    fprintf(stderr, "[mistic] join_tc KP=%d NS=%d dyn=%zu occupancy=%d grid=%u units=%llu\n", KP, NS, dyn, occ, grid,
            (unsigned long long)T.n_units);
  k_join_tc<KP, NS, G><<<grid, TC_THREADS2, dyn, h->stream>>>(P, T);
  launched(h, "join_tc");
}

}  // namespace

namespace join {

int tc_kp(uint32_t d) { return (int)(((d + 2) + 15) / 16 * 16); }
// Home rows per tensor-core unit: G chunks of 128 share each converted
// candidate tile (G = 2 while the operands leave room for two CTAs per SM).
uint32_t tc_rows(uint32_t d) { return tc_kp(d) <= 32 ? 2 * TM : TM; }
bool tc_supported(uint32_t d) { return tc_kp(d) <= 128; }

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
    default: throw Error(MISTIC_ERR_INTERNAL, "unsupported tensor-core K");
  }
}

}  // namespace join
}  // namespace mistic
