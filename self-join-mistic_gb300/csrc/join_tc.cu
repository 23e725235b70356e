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

#include "internal.cuh"

namespace mistic {
namespace {

constexpr int TM = 128;          // home rows per tile (MMA M)
constexpr int TN = 128;          // candidate columns per tile (MMA N)
constexpr int TC_THREADS = 256;  // 8 warps
constexpr int WIN = 256;         // neighbour bins per candidate window
constexpr long long kWaitLimit = 1ll << 26;
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

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t phase) {
  uint32_t done = 0;
  for (long long it = 0; it < kWaitLimit && !done; ++it) {
    asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
                 : "=r"(done)
                 : "r"(bar), "r"(phase));
  }
  return done != 0;
}

__device__ __forceinline__ void tmem_ld32(uint32_t taddr, uint32_t (&v)[32]) {
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
        "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15]),
        "=r"(v[16]), "=r"(v[17]), "=r"(v[18]), "=r"(v[19]), "=r"(v[20]), "=r"(v[21]), "=r"(v[22]), "=r"(v[23]),
        "=r"(v[24]), "=r"(v[25]), "=r"(v[26]), "=r"(v[27]), "=r"(v[28]), "=r"(v[29]), "=r"(v[30]), "=r"(v[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;");
}

__device__ __forceinline__ uint32_t pack_bf16(float a, float b) {
  __nv_bfloat162 v = __floats2bfloat162_rn(a, b);
  return *reinterpret_cast<uint32_t*>(&v);
}

// Writes one augmented row (hi part when `lo_part` is false, else lo part)
// into the core-matrix layout.  Values: k < d: scale * (x[k] - c[k]);
// k == d: ed (or the row norm when norm_at_d); k == d+1: ed1 (or the norm
// when !norm_at_d); else 0.  Returns the FP32 norm sum_k (x[k]-c[k])^2.
template <int KP>
__device__ __forceinline__ float write_row(__nv_bfloat16* base, uint32_t r, const float* __restrict__ x,
                                           const float* c, uint32_t d, uint32_t dpad, float scale, bool norm_at_d,
                                           float other, bool lo_part) {
  float nrm = 0.f;
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
        if (k < d) {
          t = xs[i] - c[k];
          nrm = fmaf(t, t, nrm);
          t *= scale;
        }
        v[h * 4 + i] = t;
      }
    }
#pragma unroll
    for (int i = 0; i < 8; ++i) {
      const uint32_t k = kb * 8 + i;
      if (k == d) v[i] = norm_at_d ? nrm : other;
      if (k == d + 1) v[i] = norm_at_d ? other : nrm;
    }
    uint4 out;
    uint32_t* o = reinterpret_cast<uint32_t*>(&out);
#pragma unroll
    for (int i = 0; i < 4; ++i) {
      float a = v[2 * i], b = v[2 * i + 1];
      if (lo_part) {
        a -= __bfloat162float(__float2bfloat16_rn(a));
        b -= __bfloat162float(__float2bfloat16_rn(b));
      }
      o[i] = pack_bf16(a, b);
    }
    const uint32_t off = (((r >> 3) * (KP / 8) + kb) * 64) + (r & 7) * 8;  // bf16 elements
    *reinterpret_cast<uint4*>(base + off) = out;
  }
  return nrm;
}

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

struct TcShared {
  float center[128];
  float na2[TM];
  uint32_t qpos[TN];
  uint32_t w_start[WIN];
  uint32_t w_pref[WIN + 1];
  uint32_t scan_ws[8];
  unsigned long long unit;
  uint32_t w_total, w_pos, seg_next, ncols, w_nb;
  uint32_t tile_maxq;  // float bits, non-negative
  uint32_t abort_flag;
  uint32_t tmem_base;
  unsigned long long bar;
};

template <int KP>
__global__ void __launch_bounds__(TC_THREADS, 1) k_join_tc(const JoinParams P, const TcParams T) {
  extern __shared__ __align__(128) unsigned char tc_dyn[];
  __shared__ TcShared S;
  constexpr uint32_t OPB = TM * KP;  // bf16 elements per operand buffer
  __nv_bfloat16* Ahi = reinterpret_cast<__nv_bfloat16*>(tc_dyn);
  __nv_bfloat16* Alo = Ahi + OPB;
  __nv_bfloat16* Bhi = Alo + OPB;
  __nv_bfloat16* Blo = Bhi + OPB;
  float* sv = reinterpret_cast<float*>(Blo + OPB);  // 8 warps x 32 lanes x SV_STRIDE
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const float* X = (const float*)P.xs;
  const uint32_t bar = smem_u32(&S.bar);

  if (tid == 0) {
    asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;" ::"r"(bar));
    asm volatile("fence.mbarrier_init.release.cluster;");
    S.abort_flag = 0;
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&S.tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = S.tmem_base;
  constexpr uint32_t idesc = umma_idesc(TM, TN);
  constexpr uint32_t SBO = 16u * KP;
  uint32_t phase = 0;
  uint32_t band_cnt = 0, amb_cnt = 0;
  bool mma_pending = false;

  for (;;) {
    if (tid == 0) S.unit = atomicAdd(&T.ctr->next_unit, 1ull);
    __syncthreads();
    const unsigned long long u = S.unit;
    if (u >= T.n_units || S.abort_flag) break;
    const Unit U = T.units[u];
    const uint32_t hs = P.bstart[U.h], he = P.bstart[U.h + 1];
    const uint32_t a0 = hs + U.chunk * TM;
    const uint32_t na = min((uint32_t)TM, he - a0);
    // unit centre = first home row; A operand once per unit
    if (tid < (int)P.dpad) S.center[tid] = X[(size_t)a0 * P.dpad + tid];
    __syncthreads();
    {
      const uint32_t r = tid & (TM - 1);
      const bool lo = tid >= TM;
      const float* xr = X + (size_t)(a0 + min(r, na - 1)) * P.dpad;
      float nrm;
      if (r < na) {
        nrm = write_row<KP>(lo ? Alo : Ahi, r, xr, S.center, P.d, P.dpad, 1.f, true, 1.f, lo);
      } else {
        const uint4 z = make_uint4(0, 0, 0, 0);
        for (int kb = 0; kb < KP / 8; ++kb)
          *reinterpret_cast<uint4*>((lo ? Alo : Ahi) + (((r >> 3) * (KP / 8) + kb) * 64) + (r & 7) * 8) = z;
        nrm = 0.f;
      }
      if (!lo) S.na2[r] = nrm;
    }
    if (tid == 0) {
      S.seg_next = U.s0;
      S.w_total = 0;
      S.w_pos = 0;
    }
    __syncthreads();

    for (;;) {
      // ---- refill the candidate window when it is used up
      if (S.w_pos >= S.w_total) {
        const uint32_t sn = S.seg_next;
        if (sn >= U.s1) break;
        const uint32_t nb = min((uint32_t)WIN, U.s1 - sn);
        uint32_t st = 0, sz = 0;
        if ((uint32_t)tid < nb) {
          const uint32_t b = P.nbr[sn + tid];
          st = P.bstart[b];
          sz = P.bstart[b + 1] - st;
        }
        const uint32_t incl = warp_scan_incl(sz);
        if (lane == 31) S.scan_ws[warp] = incl;
        __syncthreads();
        uint32_t wp = 0;
        for (int w = 0; w < warp; ++w) wp += S.scan_ws[w];
        if ((uint32_t)tid < nb) {
          S.w_start[tid] = st;
          S.w_pref[tid + 1] = wp + incl;
        }
        if (tid == 0) {
          S.w_pref[0] = 0;
          S.w_pos = 0;
          S.w_nb = nb;
          S.seg_next = sn + nb;
        }
        __syncthreads();
        if (tid == 0) S.w_total = S.w_pref[nb];
        __syncthreads();
        continue;
      }
      // ---- candidate positions of this tile
      const uint32_t wpos = S.w_pos, wtot = S.w_total;
      const uint32_t ncols = min((uint32_t)TN, wtot - wpos);
      if (tid < TN) {
        uint32_t q = 0xffffffffu;
        const uint32_t rank = wpos + tid;
        if (rank < wtot) {
          int lo = 0, hi = (int)S.w_nb - 1;
          // largest j with w_pref[j] <= rank (w_pref is non-decreasing, w_pref[0] = 0)
          while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (S.w_pref[mid] <= rank) lo = mid; else hi = mid - 1;
          }
          q = S.w_start[lo] + (rank - S.w_pref[lo]);
        }
        S.qpos[tid] = q;
      }
      if (tid == 0) {
        S.tile_maxq = 0;
        S.ncols = ncols;
      }
      __syncthreads();
      // ---- B operand: candidate rows (threads 0..127 hi, 128..255 lo)
      {
        const uint32_t r = tid & (TN - 1);
        const bool lo = tid >= TN;
        const uint32_t q = S.qpos[r];
        float nrm = 0.f;
        if (r < ncols) {
          nrm = write_row<KP>(lo ? Blo : Bhi, r, X + (size_t)q * P.dpad, S.center, P.d, P.dpad, -2.f, false,
                              1.f, lo);
        } else {
          const uint4 z = make_uint4(0, 0, 0, 0);
          for (int kb = 0; kb < KP / 8; ++kb)
            *reinterpret_cast<uint4*>((lo ? Blo : Bhi) + (((r >> 3) * (KP / 8) + kb) * 64) + (r & 7) * 8) = z;
        }
        if (!lo) {
          float m = nrm;
#pragma unroll
          for (int o = 16; o; o >>= 1) m = fmaxf(m, __shfl_xor_sync(FULL_MASK, m, o));
          if (lane == 0) atomicMax(&S.tile_maxq, __float_as_uint(m));
        }
      }
      asm volatile("fence.proxy.async.shared::cta;");
      __syncthreads();
      // ---- MMAs: D = Ahi.Bhi + Ahi.Blo + Alo.Bhi over KP/16 K steps
      if (tid == 0) {
        asm volatile("tcgen05.fence::after_thread_sync;");
        const uint32_t ah = smem_u32(Ahi), al = smem_u32(Alo), bh = smem_u32(Bhi), bl = smem_u32(Blo);
#pragma unroll
        for (int ks = 0; ks < KP / 16; ++ks) {
          const uint32_t o = ks * 256;
          mma_bf16(tbase, umma_desc(ah + o, SBO), umma_desc(bh + o, SBO), idesc, ks > 0 ? 1u : 0u);
          mma_bf16(tbase, umma_desc(ah + o, SBO), umma_desc(bl + o, SBO), idesc, 1u);
          mma_bf16(tbase, umma_desc(al + o, SBO), umma_desc(bh + o, SBO), idesc, 1u);
        }
        asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(bar));
      }
      mma_pending = true;
      // every thread waits; the outcome is made block-uniform before branching
      const bool ok = __syncthreads_and(mbar_wait(bar, phase) ? 1 : 0) != 0;
      phase ^= 1u;
      if (!ok) {
        if (tid == 0) S.abort_flag = 1u;
        break;
      }
      mma_pending = false;
      asm volatile("tcgen05.fence::after_thread_sync;");
      // ---- epilogue: warp w reads TMEM lanes 32*(w%4).., columns 64*(w/4)..
      {
        const uint32_t row = 32 * (warp & 3) + lane;
        const uint32_t a_sorted = a0 + row;
        const bool row_ok = row < na;
        // per-row thresholds for this tile (FP32, conservative)
        const float ra = sqrtf(S.na2[row] * T.ginf);
        const float rq = sqrtf(__uint_as_float(S.tile_maxq) * T.ginf);
        const float rs = ra + rq;
        const float delta = T.uR2 + T.u1 * rs;
        float E = (T.kappa * rs * rs + delta * (2.f * T.Dp + delta)) * 1.001f;
        float tlo, thi;
        if (!(E <= T.cap)) {
          tlo = -1.f;
          thi = INFINITY;
        } else {
          tlo = T.eps2_lo - E;
          tlo -= fabsf(tlo) * 1e-6f;  // round the bound outward
          thi = T.eps2_hi + E;
          thi += fabsf(thi) * 1e-6f;
        }
        float* my_sv = sv + (size_t)(warp * 32 + lane) * SV_STRIDE;
        for (int cc = 0; cc < 2; ++cc) {
          const uint32_t c0 = 64 * (warp >> 2) + 32 * cc;
          uint32_t v[32];
          tmem_ld32(tbase + ((uint32_t)(32 * (warp & 3)) << 16) + c0, v);
          uint32_t m = 0;
#pragma unroll
          for (int j = 0; j < 32; ++j) m |= (__uint_as_float(v[j]) <= thi ? 1u : 0u) << j;
          const uint32_t nvalid = ncols > c0 ? min(32u, ncols - c0) : 0u;
          m &= nvalid >= 32 ? FULL_MASK : ((1u << nvalid) - 1u);
          if (!row_ok) m = 0;
          uint32_t acc_bits = 0;
          if (__any_sync(FULL_MASK, m != 0)) {
            if (m) {
#pragma unroll
              for (int j = 0; j < 32; j += 4)
                *reinterpret_cast<float4*>(my_sv + j) =
                    make_float4(__uint_as_float(v[j]), __uint_as_float(v[j + 1]), __uint_as_float(v[j + 2]),
                                __uint_as_float(v[j + 3]));
              uint32_t bits = m;
              while (bits) {
                const int j = __ffs(bits) - 1;
                bits &= bits - 1;
                const uint32_t q = S.qpos[c0 + j];
                if (q >= hs && q < he && q <= a_sorted) continue;  // home bin: only a < q
                const float s = my_sv[j];
                if (s <= tlo) {
                  acc_bits |= 1u << j;
                } else {
                  const double sd = exact_sqdist_tc(P, P.ids[a_sorted], P.ids[q]);
                  ++band_cnt;
                  if (fabs(sd - P.eps2) <= P.amb) ++amb_cnt;
                  if (sd <= P.eps2) acc_bits |= 1u << j;
                }
              }
            }
          }
          // warp-aggregated emission of this lane's accepted columns
          const uint32_t cnt = __popc(acc_bits);
          const uint32_t incl = warp_scan_incl(cnt);
          const uint32_t total = __shfl_sync(FULL_MASK, incl, 31);
          if (total) {
            unsigned long long basep = 0;
            if (lane == 31) basep = atomicAdd(&P.ctr->pairs, (unsigned long long)total);
            basep = __shfl_sync(FULL_MASK, basep, 31);
            if (P.pairs && cnt) {
              unsigned long long pos = basep + incl - cnt;
              const uint32_t ia = P.ids[a_sorted];
              uint32_t bits = acc_bits;
              while (bits) {
                const int j = __ffs(bits) - 1;
                bits &= bits - 1;
                const uint32_t iq = P.ids[S.qpos[c0 + j]];
                const uint32_t lo = ia < iq ? ia : iq, hi = ia < iq ? iq : ia;
                if (pos < P.cap) P.pairs[pos] = ((unsigned long long)lo << 32) | hi;
                ++pos;
              }
            }
          }
        }
      }
      asm volatile("tcgen05.fence::before_thread_sync;");
      __syncthreads();
      if (tid == 0) S.w_pos = wpos + TN;
      __syncthreads();
    }
    __syncthreads();
    if (S.abort_flag) break;
  }
  // drain: an MMA whose wait expired may still be in flight; wait once more
  // (bounded) before releasing tensor memory.
  if (mma_pending) mbar_wait(bar, phase ^ 1u);
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tbase));
  if (tid == 0 && S.abort_flag) atomicExch(&P.ctr->error, 1ull);
  // counters (the pair count itself was added per warp during emission)
  const uint32_t bt = __shfl_sync(FULL_MASK, warp_scan_incl(band_cnt), 31);
  const uint32_t at = __shfl_sync(FULL_MASK, warp_scan_incl(amb_cnt), 31);
  if (lane == 0) {
    if (bt) atomicAdd(&P.ctr->band, (unsigned long long)bt);
    if (at) atomicAdd(&P.ctr->ambiguous, (unsigned long long)at);
  }
}

template <int KP>
void launch_tc(mistic_handle_s* h, const JoinParams& P, const TcParams& T) {
  const size_t dyn = 4 * (size_t)TM * KP * sizeof(__nv_bfloat16) + (size_t)8 * 32 * SV_STRIDE * sizeof(float);
  MCK(cudaFuncSetAttribute(k_join_tc<KP>, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)dyn));
  int per_sm = 0;
  MCK(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, k_join_tc<KP>, TC_THREADS, dyn));
  if (per_sm < 1) throw Error(MISTIC_ERR_TOO_LARGE, "tensor-core join does not fit on an SM");
  per_sm = std::min(per_sm, 4);  // 128 TMEM columns per CTA, 512 per SM
  const unsigned grid = (unsigned)std::min<unsigned long long>((unsigned long long)per_sm * h->sms, T.n_units);
  k_join_tc<KP><<<grid, TC_THREADS, dyn, h->stream>>>(P, T);
  launched(h, "join_tc");
}

}  // namespace

namespace join {

int tc_kp(uint32_t d) { return (int)(((d + 2) + 15) / 16 * 16); }
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
