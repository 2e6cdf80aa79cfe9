// BF16 tensor-core GEMM on the 5th-generation tensor cores (tcgen05, TMEM
// accumulators) for the ROM autoencoder:
//     C[M x N] = A[M x K] * B[N x K]^T   (+ bias[N], optional ELU)
// A and B are row-major bf16 with K contiguous ("K-major" for both operands),
// accumulation in fp32 in tensor memory.
//
// Structure (one CTA = 128 threads computes a 128 x BN tile of C; BN = 128
// for the autoencoder's layers, BN = 16 for the decoder's thin output layer
// whose B holds the 1 + k latent columns):
//  * K is consumed in slices of 64; each slice of A (128 x 64 bf16) and of B
//    (BN x 64) is copied global -> shared with cp.async into the canonical
//    K-major layout without swizzle: 8 x 16-byte "core matrices", the two
//    core matrices adjacent in K 128 bytes apart (leading byte offset) and
//    the 8-row groups 1024 bytes apart (stride byte offset);
//  * ST shared-memory stages, ST - 1 slices in flight: while the tensor core
//    works on one slice the threads' copies of the next ones land;
//  * one elected thread issues tcgen05.mma (M = 128, N = BN, K = 16, four
//    per slice) and tcgen05.commit onto the stage's mbarrier, which tells
//    the copy threads when the stage may be overwritten;
//  * the epilogue (tile_epilogue) reads the accumulator with tcgen05.ld
//    (warp w owns TMEM lanes 32 (w % 4).. = tile rows) and either adds the
//    bias, applies ELU and stores, or stores split-K partial sums, or forms
//    the output layer's squared-error gradient, or (CTAs of eight warps)
//    applies Adam to the weights whose gradient the tile is.
// Three kernels share that epilogue: k_gemm_tn (row-major operands),
// k_gemm_blocked (both operands pre-blocked, one bulk copy per slice, for
// long K) and, with its own epilogue, k_gemm_thin_blocked (N = 16).
// Every wait on an mbarrier is bounded by a clock budget; on expiry the CTA
// sets an error flag, skips the remaining work, frees its TMEM and returns.
#pragma once

#include <cstdint>

#include <cuda_bf16.h>

#include "tc_gemm_api.hpp"

namespace pda {
namespace tc {

constexpr int BM = 128, BN = 128, BK = 64, THREADS = 128, STAGES = 2;
constexpr int TILE_BYTES = BM * BK * 2;  // one 128-row operand slice
// dynamic shared memory of k_gemm_tn<bn, stages> (+ 1 KB alignment slack)
__host__ __device__ constexpr int smem_bytes(int bn, int stages) {
  return stages * (TILE_BYTES + bn * BK * 2) + 1024;
}
constexpr int SMEM_BYTES = smem_bytes(BN, STAGES);
// the decoder's output layer: N = 1 + k <= 16 columns, four stages
constexpr int THIN_BN = 16, THIN_STAGES = 4;
constexpr long long WAIT_CYCLES = 4000000000LL;  // ~2 s at 2 GHz

__device__ __forceinline__ uint32_t smem_addr(const void *p) {
  return static_cast<uint32_t>(__cvta_generic_to_shared(p));
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

// copy one ROWS x 64 slice (rows r0.., K columns k0..) of a row-major
// [rows x K] bf16 matrix into shared memory; rows past `rows` read as zero
template <int ROWS, int NT>
__device__ __forceinline__ void load_slice(uint32_t sdst, const __nv_bfloat16 *__restrict__ g, long rows, long K,
                                           long r0, long k0) {
  // ROWS rows x 8 chunks of 16 bytes over 128 threads
  static_assert((ROWS * 8) % NT == 0, "whole chunks per thread");
#pragma unroll
  for (int i = 0; i < ROWS * 8 / NT; ++i) {
    const int c = threadIdx.x + i * NT;
    const int r = c >> 3, kc = c & 7;
    const long gr = r0 + r;
    const bool valid = gr < rows;
    const __nv_bfloat16 *src = g + (valid ? gr : 0) * K + k0 + kc * 8;
    cp_async16(sdst + slice_offset(r, kc * 8), src, valid);
  }
}

// bytes of the Adam epilogue's staging: the fp32 tile (reusing the operand
// stages) and the bf16 transpose of the updated weights, rows of BM + 2
__host__ __device__ constexpr int adam_tile_bytes(int bn, int stages) {
  return stages * (TILE_BYTES + bn * BK * 2) > BM * bn * 4 ? stages * (TILE_BYTES + bn * BK * 2) : BM * bn * 4;
}
__host__ __device__ constexpr int adam_smem_bytes(int bn, int stages) {
  return adam_tile_bytes(bn, stages) + bn * (BM + 2) * 2 + 1024;
}

// The epilogue of one 128 x BN_ output tile whose accumulator sits in TMEM
// (columns 0..BN_-1; warp w reaches lanes 32 (w % 4).. = tile rows), after
// the CTA's last MMA completed, for CTAs of NT threads:
//  * NT = 256: the Adam update of the weights whose gradient the tile is
//    (adam.W; such CTAs serve nothing else);
//  * mse.X: the output layer's squared-error gradient (mseSlot: the CTA's
//    entry of mse.partial);
//  * partial: the raw sums of a K split (partial points at the split's
//    [M x N] slab);
//  * otherwise bias / ELU / the fp32, bf16 and pre-activation outputs.
// `stage` and `stageT` are shared memory that the Adam epilogue may use (the
// operand stages, no longer read by the tensor core, and the area past them).
// The remaining cases run with NT = 128.  All threads of the CTA call it (it
// synchronises inside).
template <int BN_, int NT>
__device__ __forceinline__ void tile_epilogue(uint32_t tmem, int KT, long M, long N, long m0, long n0,
                                              const float *__restrict__ bias, int epi, float *__restrict__ outF,
                                              __nv_bfloat16 *__restrict__ outB, float *__restrict__ preact,
                                              float *__restrict__ partial, const AdamEpi &adam, const MseEpi &mse,
                                              long mseSlot, uint8_t *stage, uint8_t *stageT) {
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  if (NT == 256) {
    // eight-warp CTAs serve the Adam epilogue only
    if (KT == 0 || !adam.W) return;
    // Adam on the gradient tile.  (1) TMEM -> shared memory, one fp32 row per
    // thread, 16-byte chunks XOR-swizzled by the row so that both the
    // row-per-thread writes and the row-per-warp reads are conflict-free;
    // (2) each warp updates whole rows with coalesced 16-byte streaming
    // accesses to W, m, v (touched once per step) and writes the bf16 copy,
    // keeping the new bf16 values transposed in shared memory; (3) the
    // transpose leaves as 128-byte row segments.
    static_assert(BN_ == 128, "the fused epilogues assume 128-column tiles");
    float4 *tile = reinterpret_cast<float4 *>(stage);
    __nv_bfloat16 *sT = reinterpret_cast<__nv_bfloat16 *>(stageT);
    constexpr int TS = BM + 2;  // row stride of the transposed bf16 tile
    // a warp reads the TMEM lanes of its sub-partition (warp % 4); with
    // eight warps, warps 4..7 take the second half of the columns
    constexpr int CW = BN_ / (NT / 128);
    const int r = (warp & 3) * 32 + lane;
    const int cBegin = (warp >> 2) * CW;
#pragma unroll 1
    for (int c0 = cBegin; c0 < cBegin + CW && n0 + c0 < N; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)((warp & 3) * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
#pragma unroll
      for (int u = 0; u < 4; ++u) {
        const int q = (c0 >> 2) + u;
        tile[r * (BN_ / 4) + (q ^ (r & 31))] =
            make_float4(__uint_as_float(v[4 * u]), __uint_as_float(v[4 * u + 1]), __uint_as_float(v[4 * u + 2]),
                        __uint_as_float(v[4 * u + 3]));
      }
    }
    __syncthreads();
    // RB rows per warp in flight: their W, m, v loads are issued together
    // (two CTAs of eight warps per SM keep about 100 KB of loads in flight)
    constexpr int NW = NT / 32, RB = 4;
    const long col = n0 + 4 * lane;
#pragma unroll 1
    for (int rb = warp; rb < BM; rb += RB * NW) {
      float4 w4[RB], m4[RB], v4[RB], g4[RB];
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        const int rr = rb + j * NW;
        const long idx = (m0 + rr) * N + col;
        if (m0 + rr < M && col < N) {
          w4[j] = __ldcs(reinterpret_cast<const float4 *>(adam.W + idx));
          m4[j] = __ldcs(reinterpret_cast<const float4 *>(adam.m + idx));
          v4[j] = __ldcs(reinterpret_cast<const float4 *>(adam.v + idx));
          g4[j] = tile[rr * (BN_ / 4) + (lane ^ (rr & 31))];
        }
      }
#pragma unroll
      for (int j = 0; j < RB; ++j) {
        const int rr = rb + j * NW;
        const long idx = (m0 + rr) * N + col;
        if (m0 + rr < M && col < N) {
          float *w = &w4[j].x, *mm = &m4[j].x, *vv = &v4[j].x;
          const float *g = &g4[j].x;
          __align__(8) __nv_bfloat16 hb[4];
#pragma unroll
          for (int e = 0; e < 4; ++e) {
            if (col + e < adam.cols) {
              w[e] = adam_update(w[e], mm[e], vv[e], g[e], adam.coef);
              hb[e] = __float2bfloat16_rn(w[e]);
            } else {
              hb[e] = __float2bfloat16_rn(0.f);
            }
            if (adam.WbT) sT[(4 * lane + e) * TS + rr] = hb[e];
          }
          __stcs(reinterpret_cast<float4 *>(adam.W + idx), w4[j]);
          __stcs(reinterpret_cast<float4 *>(adam.m + idx), m4[j]);
          __stcs(reinterpret_cast<float4 *>(adam.v + idx), v4[j]);
          const long ob = adam.blocked ? blocked_index(m0 + rr, col, N >> 6) : idx;
          *reinterpret_cast<uint2 *>(adam.Wb + ob) = *reinterpret_cast<const uint2 *>(hb);
        }
      }
    }
    if (adam.WbT) {
      __syncthreads();
#pragma unroll 1
      for (int c = warp; c < BN_; c += NW) {
        const long ncol = n0 + c;
        if (ncol >= N) break;
#pragma unroll
        for (int h = 0; h < BM / 64; ++h) {
          const int rr = 2 * lane + 64 * h;
          const long row = m0 + rr;
          if (row < M)
            *reinterpret_cast<uint32_t *>(adam.WbT + (adam.blocked ? blocked_index(ncol, row, M >> 6) : ncol * M + row)) =
                *reinterpret_cast<const uint32_t *>(sT + c * TS + rr);
        }
      }
    }
  } else if (KT > 0 && mse.X) {
    // reconstruction error of the output layer: one row (sample) per thread,
    // 16 columns per TMEM load; dY rows leave in 32-byte pieces, dY^T columns
    // as 64-byte warp segments
    static_assert(BN_ % 16 == 0, "16-column groups");
    const long row = m0 + warp * 32 + lane;
    double sq = 0.;
#pragma unroll 1
    for (int c0 = 0; c0 < BN_ && n0 + c0 < N; c0 += 16) {
      uint32_t v[16];
      const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16) + (uint32_t)c0;
      asm volatile(
          "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
          "%14, %15}, [%16];\n"
          : "=r"(v[0]), "=r"(v[1]), "=r"(v[2]), "=r"(v[3]), "=r"(v[4]), "=r"(v[5]), "=r"(v[6]), "=r"(v[7]),
            "=r"(v[8]), "=r"(v[9]), "=r"(v[10]), "=r"(v[11]), "=r"(v[12]), "=r"(v[13]), "=r"(v[14]), "=r"(v[15])
          : "r"(taddr));
      asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
      if (row < M) {
        const long base = row * N + n0 + c0;
        uint4 xr[2];
        xr[0] = reinterpret_cast<const uint4 *>(mse.X + base)[0];
        xr[1] = reinterpret_cast<const uint4 *>(mse.X + base)[1];
        const __nv_bfloat16 *x = reinterpret_cast<const __nv_bfloat16 *>(xr);
        __align__(16) __nv_bfloat16 dy[16];
#pragma unroll
        for (int j = 0; j < 16; ++j) {
          const long c = n0 + c0 + j;
          const float y = __uint_as_float(v[j]) + bias[c];
          const float d = y - __bfloat162float(x[j]);
          sq += (double)d * d;
          dy[j] = __float2bfloat16_rn(mse.gscale * d);
          mse.dYT[c * M + row] = dy[j];
        }
        if (mse.blocked) {
          const long kt = N >> 6;
          *reinterpret_cast<uint4 *>(mse.dY + blocked_index(row, n0 + c0, kt)) = reinterpret_cast<const uint4 *>(dy)[0];
          *reinterpret_cast<uint4 *>(mse.dY + blocked_index(row, n0 + c0 + 8, kt)) =
              reinterpret_cast<const uint4 *>(dy)[1];
        } else {
          reinterpret_cast<uint4 *>(mse.dY + base)[0] = reinterpret_cast<const uint4 *>(dy)[0];
          reinterpret_cast<uint4 *>(mse.dY + base)[1] = reinterpret_cast<const uint4 *>(dy)[1];
        }
      }
    }
    __shared__ double red[NT / 32];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) sq += __shfl_xor_sync(0xffffffffu, sq, o);
    if (lane == 0) red[warp] = sq;
    __syncthreads();
    if (threadIdx.x == 0) {
      double t = 0.;
      for (int w = 0; w < NT / 32; ++w) t += red[w];
      mse.partial[mseSlot] = t;
    }
  } else if (KT > 0) {
    const long row = m0 + warp * 32 + lane;
#pragma unroll 1
    for (int c0 = 0; c0 < BN_ && n0 + c0 < N; c0 += 16) {  // column groups that hold output columns
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
        float *pp = partial + row * N;
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
  if (NT == 128 && KT == 0 && partial) {
    // an empty split contributes zeros
    const long row = m0 + warp * 32 + lane;
    if (row < M)
      for (long col = n0; col < n0 + BN_ && col < N; ++col) partial[row * N + col] = 0.f;
  }
}

// K must be a multiple of 64; outF (fp32) and outB (bf16) are optional
// row-major [M x N] outputs (ldc = N); preact (optional, fp32) receives the
// value before the activation.  Split K: CTA z of gridDim.z covers K slices
// [z * kSlices, (z + 1) * kSlices) and, when `partial` is given, stores its
// raw fp32 sums to partial[z][M][N] (no epilogue; k_splitk_reduce finishes).
// Tiles: 128 rows of A (blockIdx.y) by BN_ rows of B (blockIdx.x).
template <int BN_, int ST, int NT = THREADS>
__global__ void __launch_bounds__(NT, NT == 256 ? 2 : 1)
k_gemm_tn(const __nv_bfloat16 *__restrict__ A, const __nv_bfloat16 *__restrict__ B, long M, long N, long K,
          const float *__restrict__ bias, int epi, float *__restrict__ outF, __nv_bfloat16 *__restrict__ outB,
          float *__restrict__ preact, int *__restrict__ err, int kSlices, float *__restrict__ partial,
          const AdamEpi adam, const MseEpi mse) {
  static_assert(BN_ >= 16 && BN_ <= 256 && BN_ % 16 == 0, "tcgen05 kind::f16 with M = 128: N in 16..256, step 16");
  static_assert(ST >= 2, "at least two stages");
  constexpr int B_BYTES = BN_ * BK * 2;
  constexpr int STAGE_BYTES = TILE_BYTES + B_BYTES;
  static_assert(STAGE_BYTES % 1024 == 0, "stages stay 1 KB aligned");
  // TMEM is allocated in powers of two of at least 32 columns
  constexpr uint32_t kTmemCols = BN_ <= 32 ? 32u : BN_ <= 64 ? 64u : BN_ <= 128 ? 128u : 256u;
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t mbar[ST];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  // 1 KB-aligned operand area
  const uint32_t sbase = (smem_addr(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long m0 = (long)blockIdx.y * BM, n0 = (long)blockIdx.x * BN_;

  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < ST; ++s)
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&mbar[s])) : "memory");
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t idesc = instr_desc(BM, BN_);

  const int KTall = (int)(K / BK);
  const int kBegin = (int)blockIdx.z * kSlices;
  const int KT = max(0, min(kSlices, KTall - kBegin));
  // slice s lives in stage s % ST; the MMAs of slice s are the (s / ST)-th
  // completion of that stage's mbarrier (parity (s / ST) & 1).  One cp.async
  // group per slice: the prologue commits slices 0..ST-2, iteration kt
  // commits slice kt + ST - 1 (an empty group past the end), so waiting until
  // at most ST - 1 groups are pending leaves slices 0..kt complete.
  auto stage_a = [&](int slice) { return sbase + (uint32_t)((slice % ST) * STAGE_BYTES); };
  auto load = [&](int slice) {
    load_slice<BM, NT>(stage_a(slice), A, M, K, m0, (long)(kBegin + slice) * BK);
    load_slice<BN_, NT>(stage_a(slice) + TILE_BYTES, B, N, K, n0, (long)(kBegin + slice) * BK);
  };
#pragma unroll 1
  for (int p = 0; p < ST - 1; ++p) {
    if (p < KT) load(p);
    asm volatile("cp.async.commit_group;\n" ::: "memory");
  }
#pragma unroll 1
  for (int kt = 0; kt < KT; ++kt) {
    const int nx = kt + ST - 1;
    if (nx < KT) {
      if (nx >= ST) {
        // the MMAs that read this stage (slice nx - ST) must be done
        if (!mbar_wait(smem_addr(&mbar[nx % ST]), (uint32_t)(((nx - ST) / ST) & 1))) abort_flag = 1;
        __syncthreads();
        if (abort_flag) break;
      }
      load(nx);
    }
    asm volatile("cp.async.commit_group;\n" ::: "memory");
    asm volatile("cp.async.wait_group %0;\n" ::"n"(ST - 1) : "memory");
    asm volatile("fence.proxy.async.shared::cta;\n" ::: "memory");
    __syncthreads();
    const uint32_t sA = stage_a(kt), sB = sA + TILE_BYTES;
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
                       smem_addr(&mbar[kt % ST]))
                   : "memory");
    }
  }
  // no copy may still be landing in shared memory when the CTA exits
  asm volatile("cp.async.wait_all;\n" ::: "memory");
  // wait for the last commit (it covers every earlier MMA of this thread)
  if (!abort_flag && KT > 0) {
    const int last = KT - 1;
    if (!mbar_wait(smem_addr(&mbar[last % ST]), (uint32_t)((last / ST) & 1))) abort_flag = 1;
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");

  if (!abort_flag) {
    uint8_t *sgen = smem_raw + (sbase - smem_addr(smem_raw));
    tile_epilogue<BN_, NT>(tmem, KT, M, N, m0, n0, bias, epi, outF, outB, preact,
                       partial ? partial + (long)blockIdx.z * M * N : nullptr, adam, mse,
                       (long)blockIdx.y * gridDim.x + blockIdx.x, sgen, sgen + adam_tile_bytes(BN_, ST));
  }
  if (abort_flag && threadIdx.x == 0) atomicExch(err, 1);
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// ---------------------------------------------------------------------------
// Thin GEMM on pre-blocked operands, for a constant wide operand streamed
// once per call (the ROM decoder's output layer, N = 16):
//   partial[z][M][16] = sum over the K slices of split z of A B^T,
// A blocked as Ablk[tile][slice] = the 128 x 64 bf16 slice of rows
// 128 tile.. in the canonical K-major no-swizzle layout (16 KB, rows past M
// zero) and B as Bblk[slice] = its 16 x 64 slice in the same layout (2 KB).
// Each slice is then one contiguous block: thread 0 moves it with one bulk
// copy (cp.async.bulk, the Tensor Memory Accelerator), counted on the stage's
// `full` mbarrier by its bytes, issues the MMAs once it lands and commits them
// to the stage's `empty` mbarrier, which frees the stage for slice kt + ST.
// A CTA's slices are consecutive blocks (one sequential stream per CTA).
// Every wait is bounded; on expiry the CTA flags the error, waits (bounded)
// for the copies it issued and returns.
// ---------------------------------------------------------------------------
constexpr int BLK_A_BYTES = BM * BK * 2, BLK_B_BYTES = THIN_BN * BK * 2;
__host__ __device__ constexpr int blocked_smem_bytes(int stages) {
  return stages * (BLK_A_BYTES + BLK_B_BYTES) + 1024;
}

__device__ __forceinline__ void bulk_g2s(uint32_t dst, const void *src, uint32_t bytes, uint32_t bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];\n" ::"r"(dst),
               "l"(src), "r"(bytes), "r"(bar)
               : "memory");
}
__device__ __forceinline__ void mbar_expect_tx(uint32_t bar, uint32_t bytes) {
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 _, [%0], %1;\n" ::"r"(bar), "r"(bytes) : "memory");
}

template <int ST>
__global__ void __launch_bounds__(THREADS)
k_gemm_thin_blocked(const __nv_bfloat16 *__restrict__ Ablk, const __nv_bfloat16 *__restrict__ Bblk, long M, int KT,
                    int kSlices, float *__restrict__ partial, int *__restrict__ err, const ThinDecode dec) {
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[ST], empty[ST];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  constexpr int STAGE = BLK_A_BYTES + BLK_B_BYTES;
  constexpr uint32_t kTmemCols = 32;
  const uint32_t sbase = (smem_addr(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  const long m0 = (long)blockIdx.x * BM;
  const int kBegin = (int)blockIdx.y * kSlices;
  const int KTc = max(0, min(kSlices, KT - kBegin));
  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < ST; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&full[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&empty[s])) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t idesc = instr_desc(BM, THIN_BN);
  const uint8_t *Ab = reinterpret_cast<const uint8_t *>(Ablk) + ((long)blockIdx.x * KT + kBegin) * BLK_A_BYTES;
  const uint8_t *Bb = reinterpret_cast<const uint8_t *>(Bblk) + (long)kBegin * BLK_B_BYTES;
  if (threadIdx.x == 0) {
    int issued = 0;  // slices whose copies were issued
    auto issue = [&](int slice) {
      const int st = slice % ST;
      const uint32_t sA = sbase + (uint32_t)(st * STAGE);
      mbar_expect_tx(smem_addr(&full[st]), (uint32_t)STAGE);
      bulk_g2s(sA, Ab + (long)slice * BLK_A_BYTES, BLK_A_BYTES, smem_addr(&full[st]));
      bulk_g2s(sA + BLK_A_BYTES, Bb + (long)slice * BLK_B_BYTES, BLK_B_BYTES, smem_addr(&full[st]));
      issued = slice + 1;
    };
    for (int p = 0; p < ST && p < KTc; ++p) issue(p);
    bool ok = true;
    for (int kt = 0; kt < KTc && ok; ++kt) {
      const int st = kt % ST;
      const uint32_t par = (uint32_t)((kt / ST) & 1);
      if (!mbar_wait(smem_addr(&full[st]), par)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t sA = sbase + (uint32_t)(st * STAGE), sB = sA + BLK_A_BYTES;
#pragma unroll
      for (int s = 0; s < BK / 16; ++s) {
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
                       smem_addr(&empty[st]))
                   : "memory");
      const int nx = kt + ST;
      if (nx < KTc) {
        // the stage is free once this slice's MMAs are done
        if (!mbar_wait(smem_addr(&empty[st]), par)) {
          ok = false;
          break;
        }
        issue(nx);
      }
    }
    if (ok && KTc > 0) {
      const int last = KTc - 1;
      if (!mbar_wait(smem_addr(&empty[last % ST]), (uint32_t)((last / ST) & 1))) ok = false;
    }
    if (!ok) {
      abort_flag = 1;
      // let the copies already issued land before the CTA's shared memory is released
      for (int sl = max(0, issued - ST); sl < issued; ++sl) mbar_wait(smem_addr(&full[sl % ST]), (uint32_t)((sl / ST) & 1));
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (!abort_flag) {
    const long row = m0 + warp * 32 + lane;
    uint32_t r[16];
    const uint32_t taddr = tmem + ((uint32_t)(warp * 32) << 16);
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, "
        "%14, %15}, [%16];\n"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
        : "r"(taddr));
    asm volatile("tcgen05.wait::ld.sync.aligned;\n" ::: "memory");
    if (row < M && dec.y) {
      // the decoder's output row (one K split: KTc covers all of K)
      const double sc = dec.scale[row];
      dec.y[row] = dec.uref[row] + sc * (double)(__uint_as_float(r[0]) + dec.b3[row]);
#pragma unroll
      for (int j = 0; j < 15; ++j)
        if (j < dec.K) dec.D[row * dec.K + j] = sc * (double)__uint_as_float(r[1 + j]);
    } else if (row < M) {
      float *pp = partial + ((long)blockIdx.y * M + row) * THIN_BN;
#pragma unroll
      for (int j = 0; j < 16; ++j) pp[j] = KTc > 0 ? __uint_as_float(r[j]) : 0.f;
    }
  } else if (threadIdx.x == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// ---------------------------------------------------------------------------
// GEMM on blocked operands for long K (the autoencoder's wide layers):
//   C = A B^T, A blocked [M / 128][K / 64] and B blocked [N / 128][K / 64]
//   (blocked_index: each 128 x 64 bf16 slice one contiguous 16 KB block).
// A CTA reads its slices of A and B as two sequential streams of 16 KB bulk
// copies (cp.async.bulk), counted by bytes on the stage's `full` mbarrier;
// one thread issues the copies and the MMAs (M = N = 128, K = 16) and
// commits each slice's MMAs to the stage's `empty` mbarrier, which frees the
// stage for slice kt + ST.  Row-major operands with long K read 128-byte
// pieces of rows a whole row apart; here each CTA streams whole blocks.
// Split K as in k_gemm_tn (CTA z covers slices [z kSlices, (z + 1) kSlices)
// and stores raw sums to partial[z]).  Every wait is bounded; on expiry the
// CTA flags the error, waits (bounded) for the copies it issued and returns.
// The epilogue is tile_epilogue (no Adam: weight gradients have short K).
// ---------------------------------------------------------------------------
constexpr int BLK_SLICE_BYTES = BM * BK * 2;
__host__ __device__ constexpr int blocked_gemm_smem_bytes(int stages) { return stages * 2 * BLK_SLICE_BYTES + 1024; }

template <int ST>
__global__ void __launch_bounds__(THREADS)
k_gemm_blocked(const __nv_bfloat16 *__restrict__ Ablk, const __nv_bfloat16 *__restrict__ Bblk, long M, long N,
               int KT, int kSlices, const float *__restrict__ bias, int epi, float *__restrict__ outF,
               __nv_bfloat16 *__restrict__ outB, float *__restrict__ preact, int *__restrict__ err,
               float *__restrict__ partial, const MseEpi mse) {
  static_assert(ST >= 2, "at least two stages");
  extern __shared__ __align__(1024) uint8_t smem_raw[];
  __shared__ __align__(8) uint64_t full[ST], empty[ST];
  __shared__ uint32_t tmem_slot;
  __shared__ int abort_flag;
  constexpr int STAGE = 2 * BLK_SLICE_BYTES;
  constexpr uint32_t kTmemCols = BN;
  const uint32_t sbase = (smem_addr(smem_raw) + 1023u) & ~1023u;
  const int warp = threadIdx.x >> 5;
  const long m0 = (long)blockIdx.y * BM, n0 = (long)blockIdx.x * BN;
  const int kBegin = (int)blockIdx.z * kSlices;
  const int KTc = max(0, min(kSlices, KT - kBegin));
  if (threadIdx.x == 0) {
    abort_flag = 0;
    for (int s = 0; s < ST; ++s) {
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&full[s])) : "memory");
      asm volatile("mbarrier.init.shared::cta.b64 [%0], 1;\n" ::"r"(smem_addr(&empty[s])) : "memory");
    }
    asm volatile("fence.mbarrier_init.release.cluster;\n" ::: "memory");
  }
  if (warp == 0) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;\n" ::"r"(smem_addr(&tmem_slot)),
                 "r"(kTmemCols)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;\n" ::: "memory");
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  const uint32_t tmem = tmem_slot;
  constexpr uint32_t idesc = instr_desc(BM, BN);
  const uint8_t *Ab = reinterpret_cast<const uint8_t *>(Ablk) + ((long)blockIdx.y * KT + kBegin) * BLK_SLICE_BYTES;
  const uint8_t *Bb = reinterpret_cast<const uint8_t *>(Bblk) + ((long)blockIdx.x * KT + kBegin) * BLK_SLICE_BYTES;
  if (threadIdx.x == 0) {
    int issued = 0;  // slices whose copies were issued
    auto issue = [&](int slice) {
      const int st = slice % ST;
      const uint32_t sA = sbase + (uint32_t)(st * STAGE);
      mbar_expect_tx(smem_addr(&full[st]), (uint32_t)STAGE);
      bulk_g2s(sA, Ab + (long)slice * BLK_SLICE_BYTES, BLK_SLICE_BYTES, smem_addr(&full[st]));
      bulk_g2s(sA + BLK_SLICE_BYTES, Bb + (long)slice * BLK_SLICE_BYTES, BLK_SLICE_BYTES, smem_addr(&full[st]));
      issued = slice + 1;
    };
    for (int p = 0; p < ST && p < KTc; ++p) issue(p);
    bool ok = true;
    for (int kt = 0; kt < KTc && ok; ++kt) {
      const int st = kt % ST;
      const uint32_t par = (uint32_t)((kt / ST) & 1);
      if (!mbar_wait(smem_addr(&full[st]), par)) {
        ok = false;
        break;
      }
      asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
      const uint32_t sA = sbase + (uint32_t)(st * STAGE), sB = sA + BLK_SLICE_BYTES;
#pragma unroll
      for (int s = 0; s < BK / 16; ++s) {
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
                       smem_addr(&empty[st]))
                   : "memory");
      const int nx = kt + ST;
      if (nx < KTc) {
        // the stage is free once this slice's MMAs are done
        if (!mbar_wait(smem_addr(&empty[st]), par)) {
          ok = false;
          break;
        }
        issue(nx);
      }
    }
    if (ok && KTc > 0) {
      const int last = KTc - 1;
      if (!mbar_wait(smem_addr(&empty[last % ST]), (uint32_t)((last / ST) & 1))) ok = false;
    }
    if (!ok) {
      abort_flag = 1;
      // let the copies already issued land before the CTA's shared memory is released
      for (int sl = max(0, issued - ST); sl < issued; ++sl) mbar_wait(smem_addr(&full[sl % ST]), (uint32_t)((sl / ST) & 1));
    }
  }
  __syncthreads();
  asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
  if (!abort_flag) {
    uint8_t *sgen = smem_raw + (sbase - smem_addr(smem_raw));
    tile_epilogue<BN, THREADS>(tmem, KTc, M, N, m0, n0, bias, epi, outF, outB, preact,
                      partial ? partial + (long)blockIdx.z * M * N : nullptr, AdamEpi{}, mse,
                      (long)blockIdx.y * gridDim.x + blockIdx.x, sgen, nullptr);
  } else if (threadIdx.x == 0) {
    atomicExch(err, 1);
  }
  asm volatile("tcgen05.fence::before_thread_sync;\n" ::: "memory");
  __syncthreads();
  if (warp == 0) {
    asm volatile("tcgen05.fence::after_thread_sync;\n" ::: "memory");
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;\n" ::"r"(tmem), "r"(kTmemCols) : "memory");
  }
}

// fp32 [R x C] -> bf16 blocked operand: trans = 0 the operand [R x C]
// (K = C), trans = 1 its transpose [C x R] (K = R); one 16-byte chunk (8
// consecutive K entries of one operand row) per thread; R and C multiples of 64
__global__ void k_to_bf16_blocked(const float *__restrict__ W, long R, long C, int trans,
                                  __nv_bfloat16 *__restrict__ out) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long rows = trans ? C : R, K = trans ? R : C;
  if (i >= rows * (K / 8)) return;
  const long r = i / (K / 8), k0 = (i % (K / 8)) * 8;
  __align__(16) __nv_bfloat16 v[8];
#pragma unroll
  for (int e = 0; e < 8; ++e) v[e] = __float2bfloat16_rn(trans ? W[(k0 + e) * C + r] : W[r * C + k0 + e]);
  *reinterpret_cast<uint4 *>(out + blocked_index(r, k0, K >> 6)) = *reinterpret_cast<const uint4 *>(v);
}

// row-major [M x K] bf16 -> the blocked layout of k_gemm_thin_blocked's A
// (rows = 128-row tiles, zero past M; `rowsPerSlice` 128 for A, 16 for B
// with M <= 16): one 16-byte chunk per thread
__global__ void k_block_operand(const __nv_bfloat16 *__restrict__ W, long M, long K, int rowsPerSlice,
                                __nv_bfloat16 *__restrict__ Wb) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  const long KT = K / BK, tiles = (M + rowsPerSlice - 1) / rowsPerSlice;
  const int chunks = rowsPerSlice * (BK / 8);
  if (i >= tiles * KT * chunks) return;
  const long blk = i / chunks;
  const int c = (int)(i % chunks);
  const long t = blk / KT, sl = blk % KT;
  const int r = c >> 3, kc = c & 7;
  const long row = t * rowsPerSlice + r;
  uint4 v = make_uint4(0u, 0u, 0u, 0u);
  if (row < M) v = *reinterpret_cast<const uint4 *>(W + row * K + sl * BK + kc * 8);
  *reinterpret_cast<uint4 *>(reinterpret_cast<uint8_t *>(Wb) + blk * (long)rowsPerSlice * BK * 2 +
                             slice_offset(r, kc * 8)) = v;
}

// sum the split-K partials in split order, then the epilogue of k_gemm_tn;
// partial[z][M][ldp] (ldp >= N: 16 for the thin blocked GEMM)
__global__ void k_splitk_reduce(long M, long N, int splits, const float *__restrict__ partial, long ldp,
                                const float *__restrict__ bias, int epi, float *__restrict__ outF,
                                __nv_bfloat16 *__restrict__ outB, float *__restrict__ preact) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= M * N) return;
  const long row = i / N, col = i % N;
  float v = 0.f;
  for (int z = 0; z < splits; ++z) v += partial[((long)z * M + row) * ldp + col];
  if (epi != EPI_NONE) v += bias[col];
  if (preact) preact[i] = v;
  if (epi == EPI_BIAS_ELU) v = elu(v);
  if (outF) outF[i] = v;
  if (outB) outB[i] = __float2bfloat16_rn(v);
}

}  // namespace tc
}  // namespace pda
