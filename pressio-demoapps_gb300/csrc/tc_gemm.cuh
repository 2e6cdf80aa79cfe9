// BF16 tensor-core GEMM on the 5th-generation tensor cores (tcgen05, TMEM
// accumulators) for the ROM autoencoder:
//     C[M x N] = A[M x K] * B[N x K]^T   (+ bias[N], optional ELU)
// A and B are row-major bf16 with K contiguous ("K-major" for both operands),
// accumulation in fp32 in tensor memory.
//
// Structure (one CTA = 128 threads computes a 128 x 128 tile of C):
//  * K is consumed in slices of 64; each slice of A and B (128 x 64 bf16 each)
//    is copied global -> shared with cp.async into the canonical K-major
//    layout without swizzle: 8 x 16-byte "core matrices", the two core
//    matrices adjacent in K 128 bytes apart (leading byte offset) and the
//    8-row groups 1024 bytes apart (stride byte offset);
//  * two shared-memory stages: while the tensor core works on one slice the
//    threads copy the next;
//  * one elected thread issues tcgen05.mma (M = 128, N = 128, K = 16, four
//    per slice) and tcgen05.commit onto the stage's mbarrier, which tells
//    the copy threads when the stage may be overwritten;
//  * the epilogue reads the accumulator with tcgen05.ld (warp w owns TMEM
//    lanes 32w..32w+31 = tile rows), adds the bias, applies ELU and stores.
// Every wait on an mbarrier is bounded by a clock budget; on expiry the CTA
// sets an error flag, skips the remaining work, frees its TMEM and returns.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>

#include "tc_gemm_api.hpp"

namespace pda {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 64, THREADS = 128, STAGES = 2;
constexpr int TILE_BYTES = BM * BK * 2;                    // one operand slice
constexpr int SMEM_BYTES = STAGES * 2 * TILE_BYTES + 1024;  // + alignment slack
constexpr uint32_t TMEM_COLS = 128;
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
}

// byte offset of element (r, k) of a 128 x 64 bf16 slice in the canonical
// K-major no-swizzle layout
__device__ __forceinline__ uint32_t slice_offset(int r, int k) {
  return (uint32_t)((((r >> 3) << 3) + (k >> 3)) << 7) + (uint32_t)((r & 7) << 4) + (uint32_t)((k & 7) << 1);
}

// shared-memory matrix descriptor: start, leading / stride byte offsets (in
// 16-byte units), descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t smem_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo) {
  uint64_t d = (uint64_t)((saddr >> 4) & 0x3FFFu);
  d |= (uint64_t)((lbo >> 4) & 0x3FFFu) << 16;
  d |= (uint64_t)((sbo >> 4) & 0x3FFFu) << 32;
  d |= (uint64_t)1 << 46;
  return d;
}

// instruction descriptor of kind::f16: D fp32, A and B bf16, both K-major
__host__ __device__ constexpr uint32_t instr_desc(int m, int n) {
  return (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(n >> 3) << 17) | ((uint32_t)(m >> 4) << 24);
}

__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src, bool valid) {
  const int n = valid ? 16 : 0;  // 0 source bytes: the 16 bytes are zero-filled
  asm volatile("cp.async.cg.shared.global [%0], [%1], 16, %2;\n" ::"r"(dst), "l"(src), "r"(n) : "memory");
}

__device__ __forceinline__ bool mbar_wait(uint32_t bar, uint32_t parity) {
  const long long t0 = clock64();
  while (true) {
    uint32_t done;
    asm volatile(
        "{\n .reg .pred p;\n mbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\n selp.b32 %0, 1, 0, p;\n}\n"
        : "=r"(done)
        : "r"(bar), "r"(parity)
        : "memory");
    if (done) return true;
    if (clock64() - t0 > WAIT_CYCLES) return false;
  }
}

__device__ __forceinline__ float elu(float x) { return x > 0.f ? x : expm1f(x); }

// copy one 128 x 64 slice (rows r0.., K columns k0..) of a row-major
// [rows x K] bf16 matrix into shared memory; rows past `rows` read as zero
__device__ __forceinline__ void load_slice(uint32_t sdst, const __nv_bfloat16 *__restrict__ g, long rows, long K,
                                           long r0, long k0) {
  // 128 rows x 8 chunks of 16 bytes; 128 threads -> 8 chunks each
#pragma unroll
  for (int i = 0; i < 8; ++i) {
    const int c = threadIdx.x + i * THREADS;
    const int r = c >> 3, kc = c & 7;
    const long gr = r0 + r;
    const bool valid = gr < rows;
    const __nv_bfloat16 *src = g + (valid ? gr : 0) * K + k0 + kc * 8;
    cp_async16(sdst + slice_offset(r, kc * 8), src, valid);
  }
}

// K must be a multiple of 64; outF (fp32) and outB (bf16) are optional
// row-major [M x N] outputs (ldc = N); preact (optional, fp32) receives the
// value before the activation.  Split K: CTA z of gridDim.z covers K slices
// [z * kSlices, (z + 1) * kSlices) and, when `partial` is given, stores its
// raw fp32 sums to partial[z][M][N] (no epilogue; k_splitk_reduce finishes).
__global__ void __launch_bounds__(THREADS)
k_gemm_tn(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B, long M, long N, long K,
          const float *__restrict__ bias, int epi, float *__restrict__ outF, __nv_bfloat16 *__restrict__ outB,
          float *__restrict__ preact, int *__restrict__ err, int kSlices, float *__restrict__ partial) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t mbar[STAGES];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  // 1 KB-aligned operand area
  const uint32_t sbase = (smem_addr(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long m0 = (long)blockIdx.y * BM, n0 = (long)blockIdx.x * BN;

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < STAGES; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&mbar[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&tmem_slot)),
                 "r"(TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t idesc = instr_desc(BM, BN);

  const int KTall = (int)(K / BK);
  const int kBegin = (int)blockIdx.z * kSlices;
  const int KT = max(0, min(kSlices, KTall - kBegin));
  for (int kt = 0; kt < KT; ++kt) {
    const int st = kt & 1;
    const uint32_t sA = sbase + (uint32_t)(st * 2 * TILE_BYTES), sB = sA + TILE_BYTES;
    if (kt >= STAGES) {
      // the MMAs that read this stage two slices ago must be done
      if (!mbar_wait(smem_addr(&mbar[st]), (uint32_t)(((kt - STAGES) >> 1) & 1))) abort_flag = 1;
      __syncthreads();
      if (abort_flag) break;
    }
    load_slice(sA, A, M, K, m0, (long)(kBegin + kt) * BK);
    load_slice(sB, B, N, K, n0, (long)(kBegin + kt) * BK);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group 0;\n" ::: "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    if (threadIdx.x == 0) {
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
#pragma unroll
      for (int s = 0; s < BK / 16; ++s) {
        // K slice s: core matrices 2s, 2s+1 along K
        const uint64_t ad = smem_desc(sA + (uint32_t)(s * 256), 128u, 1024u);
        const uint64_t bd = smem_desc(sB + (uint32_t)(s * 256), 128u, 1024u);
        const uint32_t acc = (kt > 0 || s > 0) ? 1u : 0u;
        asm volatile(
            "{\n .reg .pred p;\n setp.ne.b32 p, %4, 0;\n"
            " tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}\n" ::"r"(tmem),
            "l"(ad), "l"(bd), "r"(idesc), "r"(acc)
            : "memory");
      }
      asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];\n" ::"r"(
                       smem_addr(&mbar[st]))
                   : "memory");
    }
  }
  // wait for the last commit (it covers every earlier MMA of this thread)
  if (!abort_flag && KT > 0) {
    const int last = KT - 1;
    if (!mbar_wait(smem_addr(&mbar[last & 1]), (uint32_t)((last >> 1) & 1))) abort_flag = 1;
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

  if (!abort_flag && KT > 0) {
    const long row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN && n0 + c0 < N; c0 += 16) {  // column groups that hold output columns
      uint32_t r[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];\n"
          : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
            "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < M && partial) {
        float *pp = partial + (long)blockIdx.z * M * N + row * N;
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const long col = n0 + c0 + j;
          if (col < N) pp[col] = __uint_as_float(r[j]);
        }
      } else if (row < M) {
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const long col = n0 + c0 + j;
          if (col < N) {
            float v = __uint_as_float(r[j]);
            if (epi != EPI_NONE) v += bias[col];
            if (preact) preact[row * N + col] = v;
            if (epi == EPI_BIAS_ELU) v = elu(v);
            if (outF) outF[row * N + col] = v;
            if (outB) outB[row * N + col] = __float2bfloat16_rn(v);
          }
        }
      }
    }
  }
  if (!abort_flag && KT == 0 && partial) {
    // an empty split contributes zeros
    const long row = m0 + warp * 32 + lane;
    if (row < M)
      for (long col = n0; col < n0 + BN && col < N; ++col) partial[(long)blockIdx.z * M * N + row * N + col] = 0.f;
  }
  if (abort_flag && threadIdx.x == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(TMEM_COLS) : "memory");
  }
}

// sum the split-K partials in split order, then the epilogue of k_gemm_tn
__global__ void k_splitk_reduce(long M, long N, int splits, const float *__restrict__ partial,
                                const float *__restrict__ bias, int epi, float *__restrict__ outF,
                                __nv_bfloat16 *__restrict__ outB, float *__restrict__ preact) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * N) return;
  float v = 0.f;
  for (int z = 0; z < splits; ++z) v += partial[(long)z * M * N + i];
  if (epi != EPI_NONE) v += bias[i % N];
  if (preact) preact[i] = v;
  if (epi == EPI_BIAS_ELU) v = elu(v);
  if (outF) outF[i] = v;
  if (outB) outB[i] = __float2bfloat16_rn(v);
}

}  // namespace tc
}  // namespace pda
