// Tensor-core Gram probe: one 128 x 128 tile D = A B^T through tcgen05.mma,
// exactly as the join kernels issue it (no-swizzle K-major core matrices,
// FP32 accumulation in tensor memory, K/16 or K/8 instructions chained with
// the accumulate flag).
//
// It has no counterpart in the reference.  It exists so that the error
// allowance the joins' band bound assumes for the tensor cores' FP32
// accumulation (2^-19 of the sum of |products| per MMA instruction, see
// join_tc.cu) can be measured against exact products: a test feeds random
// and cancellation-heavy operands and compares D with an exact sum.
//
// Kinds: 0 = bf16 operands (kind::f16, K a multiple of 16), 1 = tf32
// operands given as FP32 bit patterns (kind::tf32, K a multiple of 8; the
// tensor core reads the top 19 bits).  K <= 256 (bf16) or 128 (tf32).  One CTA of 128 threads;
// the only wait (the MMA's completion) is bounded.
#include <cuda_bf16.h>
#include <math.h>
#include <string.h>

#include <cstdio>

#include "internal.cuh"
#include "tc_common.cuh"

namespace mistic {
namespace {

using namespace tcu;

constexpr int PM = 128, PN = 128, PKMAX = 256;

struct ProbeShared {
  unsigned long long done;
  uint32_t tmem_base;
  uint32_t abort_flag;
};

// byte offset of 16-byte chunk c of row r in a K-major no-swizzle operand of
// `row_bytes` bytes a row (8-row groups of row_bytes * 8, core matrices of
// 8 rows x 16 B, K-adjacent core matrices 128 B apart)
__device__ __forceinline__ uint32_t core_off(uint32_t r, uint32_t c, uint32_t row_bytes) {
  return ((r >> 3) * (row_bytes / 16) + c) * 128 + (r & 7) * 16;
}

__global__ void __launch_bounds__(128, 1)
    k_tc_probe(const unsigned char* __restrict__ a, const unsigned char* __restrict__ b, uint32_t row_bytes, int kind,
               uint32_t n_inst, float* __restrict__ d, uint32_t* __restrict__ status) {
  extern __shared__ __align__(128) unsigned char probe_dyn[];
  __shared__ ProbeShared S;
  unsigned char* sa = probe_dyn;
  unsigned char* sb = probe_dyn + (size_t)PM * row_bytes;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  // operands into the core-matrix layout, 16 bytes at a time
  const uint32_t chunks = row_bytes / 16;
  for (uint32_t i = tid; i < PM * chunks; i += blockDim.x) {
    const uint32_t r = i / chunks, c = i % chunks;
    *reinterpret_cast<uint4*>(sa + core_off(r, c, row_bytes)) =
        *reinterpret_cast<const uint4*>(a + (size_t)r * row_bytes + 16 * c);
    *reinterpret_cast<uint4*>(sb + core_off(r, c, row_bytes)) =
        *reinterpret_cast<const uint4*>(b + (size_t)r * row_bytes + 16 * c);
  }
  if (tid == 0) {
    mbar_init(&S.done, 1);
    S.abort_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], 128;" ::"r"(smem_u32(&S.tmem_base)));
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;");
  }
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");  // generic-proxy writes -> MMA reads
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;");
  const uint32_t tbase = S.tmem_base;
  if (tid == 0) {
    const uint32_t sbo = 8 * row_bytes;
    const uint32_t idesc = umma_idesc_fmt(PM, PN, kind == 1 ? 2u : 1u);  // TF32 : BF16
    const uint32_t a0 = smem_u32(sa), b0 = smem_u32(sb);
    for (uint32_t ks = 0; ks < n_inst; ++ks) {
      const uint32_t o = ks * 256;  // 32 bytes of K per instruction = two core matrices
      if (kind == 1)
        mma_tf32(tbase, umma_desc(a0 + o, sbo), umma_desc(b0 + o, sbo), idesc, ks > 0 ? 1u : 0u);
      else
        mma_bf16(tbase, umma_desc(a0 + o, sbo), umma_desc(b0 + o, sbo), idesc, ks > 0 ? 1u : 0u);
    }
    tc_commit(&S.done);
  }
  __syncwarp();
  const bool ok = __all_sync(FULL_MASK, wait_or_abort(&S.done, 0, &S.abort_flag, 2000000000ll));
  if (ok) {
    asm volatile("tcgen05.fence::after_thread_sync;");
    // warp w reads TMEM lanes 32w .. 32w + 31 (rows), all 128 columns
    for (uint32_t c0 = 0; c0 < PN; c0 += 32) {
      uint32_t v[32];
      tmem_ld32_nowait(tbase + ((uint32_t)(warp * 32) << 16) + c0, v);
      tmem_wait();
      const uint32_t row = warp * 32 + lane;
#pragma unroll
      for (int j = 0; j < 32; ++j) d[(size_t)row * PN + c0 + j] = __uint_as_float(v[j]);
    }
  } else if (tid == 0) {
    *status = 1;
  }
  asm volatile("tcgen05.fence::before_thread_sync;");
  __syncthreads();
  if (warp == 0) asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, 128;" ::"r"(tbase));
}

}  // namespace
}  // namespace mistic

extern "C" mistic_status mistic_tc_gram_probe(int kind, const void* a, const void* b, uint32_t K, float* d) {
  using namespace mistic;
  if (!a || !b || !d || (kind != 0 && kind != 1)) return MISTIC_ERR_INVALID_ARG;
  const uint32_t step = kind == 1 ? 8 : 16;
  if (K == 0 || K % step || K > (kind == 1 ? PKMAX / 2 : PKMAX)) return MISTIC_ERR_INVALID_ARG;
  const uint32_t esz = kind == 1 ? 4 : 2;
  const uint32_t row_bytes = K * esz;
  const size_t op_bytes = (size_t)PM * row_bytes;
  unsigned char *da = nullptr, *db = nullptr;
  float* dd = nullptr;
  uint32_t* dst = nullptr;
  mistic_status s = MISTIC_OK;
  auto ck = [&](cudaError_t e) {
    if (e != cudaSuccess && s == MISTIC_OK) {
      cudaGetLastError();
      s = e == cudaErrorMemoryAllocation ? MISTIC_ERR_OUT_OF_MEMORY : MISTIC_ERR_CUDA;
    }
    return s == MISTIC_OK;
  };
  int dev = 0;
  cudaDeviceProp p;
  if (!ck(cudaGetDevice(&dev)) || !ck(cudaGetDeviceProperties(&p, dev))) return s;
  if (p.major < 10) return MISTIC_ERR_NO_DEVICE;
  if (ck(cudaMalloc(&da, op_bytes)) && ck(cudaMalloc(&db, op_bytes)) &&
      ck(cudaMalloc(&dd, (size_t)PM * PN * sizeof(float))) && ck(cudaMalloc(&dst, sizeof(uint32_t))) &&
      ck(cudaMemcpy(da, a, op_bytes, cudaMemcpyHostToDevice)) && ck(cudaMemcpy(db, b, op_bytes, cudaMemcpyHostToDevice)) &&
      ck(cudaMemset(dst, 0, sizeof(uint32_t)))) {
    const size_t smem = 2 * op_bytes;
    if (ck(cudaFuncSetAttribute(k_tc_probe, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem))) {
      k_tc_probe<<<1, 128, smem>>>(da, db, row_bytes, kind, K / step, dd, dst);
      uint32_t hs = 0;
      if (ck(cudaGetLastError()) && ck(cudaDeviceSynchronize()) &&
          ck(cudaMemcpy(d, dd, (size_t)PM * PN * sizeof(float), cudaMemcpyDeviceToHost)) &&
          ck(cudaMemcpy(&hs, dst, sizeof hs, cudaMemcpyDeviceToHost)) && hs)
        s = MISTIC_ERR_TIMEOUT;
    }
  }
  cudaFree(da);
  cudaFree(db);
  cudaFree(dd);
  cudaFree(dst);
  return s;
}
