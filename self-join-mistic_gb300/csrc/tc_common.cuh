// Device helpers shared by the tensor-core joins (join_tc.cu: augmented K up
// to 128 in one operand tile; join_tcw.cu: long rows in K chunks).
//
// tcgen05 operands live in shared memory in the no-swizzle K-major
// core-matrix layout: a core matrix is 8 rows x 16 bytes (8 bf16), stored as
// 128 contiguous bytes; K-adjacent core matrices are LBO = 128 B apart and
// 8-row groups SBO = 16 * K bytes apart (K = the operand buffer's K extent).
#pragma once

#include <cuda_bf16.h>
#include <math.h>
#include <stdint.h>

#include "internal.cuh"

namespace mistic {
namespace tcu {

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

// Instruction descriptor: D f32, A/B of format `fmt` (1: bf16 under
// kind::f16, 2: tf32 under kind::tf32), both K-major, N x M.
__host__ __device__ constexpr uint32_t umma_idesc_fmt(int M, int N, uint32_t fmt) {
  return (1u << 4) | (fmt << 7) | (fmt << 10) | ((uint32_t)(N >> 3) << 17) | ((uint32_t)(M >> 4) << 24);
}
// kind::f16 with bf16 operands
__host__ __device__ constexpr uint32_t umma_idesc(int M, int N) { return umma_idesc_fmt(M, N, 1u); }

__device__ __forceinline__ void mma_bf16(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
      "l"(da), "l"(db), "r"(idesc), "r"(acc));
}

// kind::tf32: FP32 operands of which the tensor core reads the top 19 bits
// (the joins round them to tf32 beforehand, so nothing is dropped here)
__device__ __forceinline__ void mma_tf32(uint32_t tmem, uint64_t da, uint64_t db, uint32_t idesc, uint32_t acc) {
  asm volatile(
      "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
      " tcgen05.mma.cta_group::1.kind::tf32 [%0], %1, %2, %3, p;\n}" ::"r"(tmem),
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

__device__ __forceinline__ uint32_t warp_scan_incl(uint32_t x) {
  const int lane = threadIdx.x & 31;
#pragma unroll
  for (int o = 1; o < 32; o <<= 1) {
    const uint32_t y = __shfl_up_sync(FULL_MASK, x, o);
    if (lane >= o) x += y;
  }
  return x;
}

__device__ __forceinline__ void mbar_init(unsigned long long* b, uint32_t count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(b)), "r"(count));
}
__device__ __forceinline__ void mbar_arrive(unsigned long long* b) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0];\n}" ::"r"(smem_u32(b)) : "memory");
}
// n arrivals at once
__device__ __forceinline__ void mbar_arrive_n(unsigned long long* b, uint32_t n) {
  asm volatile("{\n .reg .b64 st;\n mbarrier.arrive.shared::cta.b64 st, [%0], %1;\n}" ::"r"(smem_u32(b)), "r"(n)
               : "memory");
}
__device__ __forceinline__ void tc_commit(unsigned long long* b) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(b))
               : "memory");
}

__device__ __forceinline__ unsigned long long global_ns() {
  unsigned long long t;
  asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
  return t;
}

// Non-blocking test of an mbarrier phase.
__device__ __forceinline__ bool mbar_ready(unsigned long long* b, uint32_t parity) {
  uint32_t done;
  asm volatile("{\n .reg .pred p;\n mbarrier.test_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(done)
               : "r"(smem_u32(b)), "r"(parity)
               : "memory");
  return done != 0;
}

// Bounded wait on an mbarrier phase.  The waiting warp is suspended by the
// hardware (try_wait with a suspend-time hint) instead of spinning, so idle
// roles leave the issue slots to the working ones.  After limit_ns of
// waiting the CTA's abort flag is raised.  Returns false if the CTA is
// aborting (now or already).
constexpr uint32_t kSuspendNs = 20000;
__device__ __forceinline__ bool wait_or_abort(unsigned long long* b, uint32_t parity, volatile uint32_t* abort_flag,
                                              long long limit_ns) {
  const uint32_t a = smem_u32(b);
  uint32_t done;
  asm volatile("{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.u32 %0, 1, 0, p;\n}"
               : "=r"(done)
               : "r"(a), "r"(parity)
               : "memory");
  if (done) return true;
  const unsigned long long t0 = global_ns();
  for (;;) {
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2, %3;\n selp.u32 %0, 1, 0, p;\n}"
        : "=r"(done)
        : "r"(a), "r"(parity), "r"(kSuspendNs)
        : "memory");
    if (done) return true;
    if (*abort_flag) return false;
    if ((long long)(global_ns() - t0) > limit_ns) {
      *abort_flag = 1u;
      return false;
    }
  }
}

// bf16 offset of the 16-byte chunk of row r and K block kb (8 bf16) in an
// operand buffer of K extent KX.
template <int KX>
__device__ __forceinline__ uint32_t chunk_off(uint32_t r, uint32_t kb) {
  return ((r >> 3) * (KX / 8) + kb) * 64 + (r & 7) * 8;
}

__device__ __forceinline__ void cp_async16(void* dst, const void* src) {
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(smem_u32(dst)), "l"(src) : "memory");
}

// Per-column threshold T(n) and accept distance dlt(n) of the tensor-core
// filter, from the unit's largest |a|^2 and this column's |q|^2 (FP32,
// rounded outward).  Returns false when the bound is too wide to decide
// anything (the column is then re-decided entirely in FP64).
__device__ __forceinline__ bool column_threshold(const TcBound& T, float ra2max, float nq2, float* tcol,
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

// v[j] without dynamic register indexing: a 5-level select tree.
__device__ __forceinline__ float pick32(const uint32_t (&v)[32], int j) {
  uint32_t t16[16], t8[8], t4[4], t2[2];
#pragma unroll
  for (int k = 0; k < 16; ++k) t16[k] = (j & 16) ? v[16 + k] : v[k];
#pragma unroll
  for (int k = 0; k < 8; ++k) t8[k] = (j & 8) ? t16[8 + k] : t16[k];
#pragma unroll
  for (int k = 0; k < 4; ++k) t4[k] = (j & 4) ? t8[4 + k] : t8[k];
#pragma unroll
  for (int k = 0; k < 2; ++k) t2[k] = (j & 2) ? t4[2 + k] : t4[k];
  return __uint_as_float((j & 1) ? t2[1] : t2[0]);
}

}  // namespace tcu
}  // namespace mistic
