// Autoencoder building blocks for the learned-manifold ROM: the tcgen05 BF16
// GEMM launcher and the elementwise / reduction kernels of training (ELU
// backward, bias gradients, transposes, MSE, Adam).
#include <algorithm>
#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "../../include/pda_gb300.h"
#include "internal.hpp"
#include "tc_gemm.cuh"

#include <string>

namespace pda {

static __device__ int g_tc_err;

// lifts the dynamic shared-memory limit of one GEMM instantiation to what
// its largest epilogue needs (a per-device function attribute, set once per
// device)
template <int BN_, int ST, int NT = tc::THREADS>
static cudaError_t gemm_attr() {
  constexpr int kMaxDev = 64;
  static bool done[kMaxDev] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev || !done[dev]) {
    const int bytes = tc::smem_bytes(BN_, ST) > tc::adam_smem_bytes(BN_, ST) ? tc::smem_bytes(BN_, ST)
                                                                              : tc::adam_smem_bytes(BN_, ST);
    e = cudaFuncSetAttribute(tc::k_gemm_tn<BN_, ST, NT>, cudaFuncAttributeMaxDynamicSharedMemorySize, bytes);
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < kMaxDev) done[dev] = true;
  }
  return cudaSuccess;
}

// one launch of k_gemm_tn (128 x 128 tiles) over all output tiles and
// `splits` K ranges of `per` slices; split-K launches (two CTAs per SM) keep
// two slices in flight per CTA (three stages), the others one (two stages,
// three CTAs per SM)
static cudaError_t launch_gemm(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                               const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact,
                               int splits, int per, float *partial, cudaStream_t s,
                               const tc::AdamEpi &adam = tc::AdamEpi{}, const tc::MseEpi &mse = tc::MseEpi{}) {
  int *err = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void **)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const dim3 grid((unsigned)((N + tc::BN - 1) / tc::BN), (unsigned)((M + tc::BM - 1) / tc::BM), (unsigned)splits);
  if (splits > 1) {
    constexpr int ST = 3;
    e = gemm_attr<tc::BN, ST>();
    if (e != cudaSuccess) return e;
    tc::k_gemm_tn<tc::BN, ST><<<grid, tc::THREADS, tc::smem_bytes(tc::BN, ST), s>>>(
        A, B, M, N, K, bias, epi, outF, outB, preact, err, per, partial, adam, mse);
  } else if (adam.W) {
    // the Adam epilogue runs eight warps: twice the rows in flight and half
    // the dependent optimizer arithmetic per warp
    constexpr int ST = tc::STAGES, NT = 2 * tc::THREADS;
    e = gemm_attr<tc::BN, ST, NT>();
    if (e != cudaSuccess) return e;
    tc::k_gemm_tn<tc::BN, ST, NT><<<grid, NT, tc::adam_smem_bytes(tc::BN, ST), s>>>(
        A, B, M, N, K, bias, epi, outF, outB, preact, err, per, partial, adam, mse);
  } else {
    constexpr int ST = tc::STAGES;
    e = gemm_attr<tc::BN, ST>();
    if (e != cudaSuccess) return e;
    tc::k_gemm_tn<tc::BN, ST><<<grid, tc::THREADS, tc::smem_bytes(tc::BN, ST), s>>>(
        A, B, M, N, K, bias, epi, outF, outB, preact, err, per, partial, adam, mse);
  }
  return cudaGetLastError();
}

cudaError_t tc_gemm_adam(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                         const tc::AdamEpi &adam, cudaStream_t s) {
  const auto misaligned = [](const void *p) { return ((uintptr_t)p & 15u) != 0; };
  if (K % tc::BK != 0 || N % 4 != 0 || M % 2 != 0 || !adam.W || !adam.m || !adam.v || !adam.Wb ||
      misaligned(adam.W) || misaligned(adam.m) || misaligned(adam.v) || ((uintptr_t)adam.Wb & 7u) != 0 ||
      ((uintptr_t)adam.WbT & 3u) != 0)
    return cudaErrorInvalidValue;
  return launch_gemm(A, B, M, N, K, nullptr, tc::EPI_NONE, nullptr, nullptr, nullptr, 1, (int)(K / tc::BK), nullptr,
                     s, adam, tc::MseEpi{});
}

cudaError_t tc_gemm_mse(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K, const float *bias,
                        const tc::MseEpi &mse, cudaStream_t s) {
  if (K % tc::BK != 0 || N % 16 != 0 || !bias || !mse.X || !mse.dY || !mse.dYT || !mse.partial ||
      ((uintptr_t)mse.X & 15u) != 0 || ((uintptr_t)mse.dY & 15u) != 0)
    return cudaErrorInvalidValue;
  return launch_gemm(A, B, M, N, K, bias, tc::EPI_BIAS, nullptr, nullptr, nullptr, 1, (int)(K / tc::BK), nullptr, s,
                     tc::AdamEpi{}, mse);
}

cudaError_t tc_gemm(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K, const float *bias,
                    int epi, float *outF, __nv_bfloat16 *outB, float *preact, cudaStream_t s) {
  return launch_gemm(A, B, M, N, K, bias, epi, outF, outB, preact, 1, (int)(K / tc::BK), nullptr, s);
}

// Same, splitting K over `splits` CTAs per output tile when the tiles alone
// would leave most SMs idle (few output tiles, long K); the partial sums go to
// `work` (splits * M * N floats) and are added in split order, so the result
// does not depend on scheduling.
cudaError_t tc_gemm_splitk(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                           const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact, float *work,
                           long workFloats, cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  const long tiles = ((N + tc::BN - 1) / tc::BN) * ((M + tc::BM - 1) / tc::BM);
  const int kt = (int)(K / tc::BK);
  int splits = 1;
  if (tiles < 2L * sms && kt >= 32) {
    splits = (int)std::min<long>((2L * sms + tiles - 1) / tiles, kt / 16);
    while (splits > 1 && (long)splits * M * N > workFloats) --splits;
  }
  if (splits <= 1) return tc_gemm(A, B, M, N, K, bias, epi, outF, outB, preact, s);
  const int per = (kt + splits - 1) / splits;
  cudaError_t e = launch_gemm(A, B, M, N, K, nullptr, tc::EPI_NONE, nullptr, nullptr, nullptr, splits, per, work, s);
  if (e != cudaSuccess) return e;
  const long total = M * N;
  tc::k_splitk_reduce<<<(unsigned)((total + 255) / 256), 256, 0, s>>>(M, N, splits, work, N, bias, epi, outF,
                                                                       outB, preact);
  return cudaGetLastError();
}

// blocked-operand GEMM: three stages (two slices in flight per CTA, two CTAs
// per SM)
cudaError_t tc_gemm_blocked(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long N, long K,
                            const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact,
                            const tc::MseEpi *mse, float *work, long workFloats, cudaStream_t s) {
  constexpr int ST = 3;
  if (K % tc::BK != 0 || (mse && (N % 16 != 0 || !bias || !mse->X || !mse->dY || !mse->dYT || !mse->partial)))
    return cudaErrorInvalidValue;
  constexpr int kMaxDev = 64;
  static bool attr[kMaxDev] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev || !attr[dev]) {
    e = cudaFuncSetAttribute(tc::k_gemm_blocked<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             tc::blocked_gemm_smem_bytes(ST));
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < kMaxDev) attr[dev] = true;
  }
  int sms = 0;
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  int *err = nullptr;
  e = cudaGetSymbolAddress((void **)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const long tiles = ((N + tc::BN - 1) / tc::BN) * ((M + tc::BM - 1) / tc::BM);
  const int kt = (int)(K / tc::BK);
  int splits = 1;
  if (!mse && work && tiles < 2L * sms && kt >= 32) {
    splits = (int)std::min<long>((2L * sms + tiles - 1) / tiles, kt / 16);
    while (splits > 1 && (long)splits * M * N > workFloats) --splits;
  }
  const int per = (kt + splits - 1) / splits;
  const dim3 grid((unsigned)((N + tc::BN - 1) / tc::BN), (unsigned)((M + tc::BM - 1) / tc::BM), (unsigned)splits);
  const tc::MseEpi me = mse ? *mse : tc::MseEpi{};
  if (splits == 1) {
    tc::k_gemm_blocked<ST><<<grid, tc::THREADS, tc::blocked_gemm_smem_bytes(ST), s>>>(
        Ablk, Bblk, M, N, kt, per, bias, epi, outF, outB, preact, err, nullptr, me);
    return cudaGetLastError();
  }
  tc::k_gemm_blocked<ST><<<grid, tc::THREADS, tc::blocked_gemm_smem_bytes(ST), s>>>(
      Ablk, Bblk, M, N, kt, per, nullptr, tc::EPI_NONE, nullptr, nullptr, nullptr, err, work, me);
  e = cudaGetLastError();
  if (e != cudaSuccess) return e;
  tc::k_splitk_reduce<<<(unsigned)((M * N + 255) / 256), 256, 0, s>>>(M, N, splits, work, N, bias, epi, outF, outB,
                                                                       preact);
  return cudaGetLastError();
}

cudaError_t tc_to_bf16_blocked(const float *W, long R, long C, int trans, __nv_bfloat16 *out, cudaStream_t s) {
  if (R % 64 != 0 || C % 64 != 0) return cudaErrorInvalidValue;
  const long n = R * C / 8;
  tc::k_to_bf16_blocked<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(W, R, C, trans, out);
  return cudaGetLastError();
}

cudaError_t tc_block_operand(const __nv_bfloat16 *W, long M, long K, int rowsPerSlice, __nv_bfloat16 *Wb,
                             cudaStream_t s) {
  if (K % tc::BK != 0 || (rowsPerSlice != tc::BM && !(rowsPerSlice == tc::THIN_BN && M <= tc::THIN_BN)))
    return cudaErrorInvalidValue;
  const long n = (M + rowsPerSlice - 1) / rowsPerSlice * (K / tc::BK) * rowsPerSlice * (tc::BK / 8);
  tc::k_block_operand<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(W, M, K, rowsPerSlice, Wb);
  return cudaGetLastError();
}

// the larger dynamic shared memory of the thin GEMM is a per-device function
// attribute, set once per device
template <int ST>
static cudaError_t thin_attr() {
  constexpr int kMaxDev = 64;
  static bool attr[kMaxDev] = {};
  int dev = 0;
  cudaError_t e = cudaGetDevice(&dev);
  if (e != cudaSuccess) return e;
  if (dev < 0 || dev >= kMaxDev || !attr[dev]) {
    e = cudaFuncSetAttribute(tc::k_gemm_thin_blocked<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                             tc::blocked_smem_bytes(ST));
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < kMaxDev) attr[dev] = true;
  }
  return cudaSuccess;
}

cudaError_t tc_gemm_thin_blocked(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long K, int splits,
                                 float *partial, cudaStream_t s) {
  constexpr int ST = tc::THIN_STAGES;
  cudaError_t e = thin_attr<ST>();
  if (e != cudaSuccess) return e;
  int *err = nullptr;
  e = cudaGetSymbolAddress((void **)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const int kt = (int)(K / tc::BK);
  splits = std::max(1, std::min(splits, kt));
  const int per = (kt + splits - 1) / splits;
  dim3 grid((unsigned)((M + tc::BM - 1) / tc::BM), (unsigned)splits);
  tc::k_gemm_thin_blocked<ST><<<grid, tc::THREADS, tc::blocked_smem_bytes(ST), s>>>(Ablk, Bblk, M, kt, per, partial,
                                                                                    err, tc::ThinDecode{});
  return cudaGetLastError();
}

cudaError_t tc_gemm_thin_prepare() { return thin_attr<tc::THIN_STAGES>(); }

cudaError_t tc_gemm_thin_decode(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long K,
                                const tc::ThinDecode &dec, cudaStream_t s) {
  constexpr int ST = tc::THIN_STAGES;
  if (!dec.y || !dec.D || !dec.b3 || !dec.uref || !dec.scale || dec.K < 1 || dec.K > 15 || K % tc::BK != 0)
    return cudaErrorInvalidValue;
  cudaError_t e = thin_attr<ST>();
  if (e != cudaSuccess) return e;
  int *err = nullptr;
  e = cudaGetSymbolAddress((void **)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const int kt = (int)(K / tc::BK);
  dim3 grid((unsigned)((M + tc::BM - 1) / tc::BM), 1u);
  tc::k_gemm_thin_blocked<ST><<<grid, tc::THREADS, tc::blocked_smem_bytes(ST), s>>>(Ablk, Bblk, M, kt, kt, nullptr,
                                                                                    err, dec);
  return cudaGetLastError();
}

// B with at most 16 rows: both operands blocked into scratch, the thin
// blocked GEMM (K split over the SMs when the row tiles are few and K long),
// then the split reduction with the epilogue
static cudaError_t tc_gemm_thin(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                                const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact,
                                cudaStream_t s) {
  int dev = 0, sms = 1;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  const long tiles = (M + tc::BM - 1) / tc::BM, kt = K / tc::BK;
  int splits = 1;
  if (tiles < 2L * sms && kt >= 32) splits = (int)std::min<long>((2L * sms + tiles - 1) / tiles, kt / 16);
  __nv_bfloat16 *Ablk = nullptr, *Bblk = nullptr;
  float *part = nullptr;
  cudaError_t e = cudaMalloc((void **)&Ablk, (size_t)tiles * tc::BM * K * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc((void **)&Bblk, (size_t)tc::THIN_BN * K * sizeof(__nv_bfloat16));
  if (e == cudaSuccess) e = cudaMalloc((void **)&part, (size_t)splits * M * tc::THIN_BN * sizeof(float));
  if (e == cudaSuccess) e = tc_block_operand(A, M, K, tc::BM, Ablk, s);
  if (e == cudaSuccess) e = tc_block_operand(B, N, K, tc::THIN_BN, Bblk, s);
  if (e == cudaSuccess) e = tc_gemm_thin_blocked(Ablk, Bblk, M, K, splits, part, s);
  if (e == cudaSuccess) {
    tc::k_splitk_reduce<<<(unsigned)((M * N + 255) / 256), 256, 0, s>>>(M, N, splits, part, tc::THIN_BN, bias, epi,
                                                                          outF, outB, preact);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  cudaFree(Ablk);
  cudaFree(Bblk);
  cudaFree(part);
  return e;
}

// 1 if any tensor-core GEMM gave up waiting since the last call; clears it
int tc_gemm_error_and_clear() {
  int h = 0;
  if (cudaMemcpyFromSymbol(&h, g_tc_err, sizeof(int)) != cudaSuccess) return -1;
  const int z = 0;
  cudaMemcpyToSymbol(g_tc_err, &z, sizeof(int));
  return h;
}

}  // namespace pda

extern "C" {

pda_status pda_tc_gemm_bf16(const void *d_A, const void *d_B, int64_t M, int64_t N, int64_t K, const float *d_bias,
                            int epilogue, float *d_outF, void *d_outB, float *d_preact, void *stream) {
  if (!d_A || !d_B || M <= 0 || N <= 0 || K <= 0 || K % pda::tc::BK != 0 || epilogue < 0 || epilogue > 2 ||
      (epilogue != 0 && !d_bias) || (!d_outF && !d_outB) ||
      ((uintptr_t)d_A & 15u) != 0 || ((uintptr_t)d_B & 15u) != 0) {
    pda::set_last_error("pda_tc_gemm_bf16: invalid argument (K must be a multiple of 64, A/B 16-byte aligned)");
    return PDA_ERR_INVALID_ARGUMENT;
  }
  cudaStream_t s = (cudaStream_t)stream;
  if (N <= pda::tc::THIN_BN) {
    const cudaError_t e = pda::tc_gemm_thin((const __nv_bfloat16 *)d_A, (const __nv_bfloat16 *)d_B, M, N, K, d_bias,
                                            epilogue, d_outF, (__nv_bfloat16 *)d_outB, d_preact, s);
    if (e != cudaSuccess) {
      pda::set_last_error(std::string("pda_tc_gemm_bf16: ") + cudaGetErrorString(e));
      return PDA_ERR_CUDA;
    }
    if (pda::tc_gemm_error_and_clear() != 0) {
      pda::set_last_error("pda_tc_gemm_bf16: a tensor-core wait timed out");
      return PDA_ERR_CUDA;
    }
    return PDA_OK;
  }
  // split-K scratch for shapes with few output tiles and a long K
  float *work = nullptr;
  const long workFloats = 32L * M * N;
  if ((K / pda::tc::BK) >= 32 && ((M + 127) / 128) * ((N + 127) / 128) < 304 &&
      cudaMalloc((void **)&work, (size_t)workFloats * sizeof(float)) != cudaSuccess) {
    work = nullptr;
    cudaGetLastError();
  }
  cudaError_t e = work ? pda::tc_gemm_splitk((const __nv_bfloat16 *)d_A, (const __nv_bfloat16 *)d_B, M, N, K, d_bias,
                                             epilogue, d_outF, (__nv_bfloat16 *)d_outB, d_preact, work, workFloats, s)
                       : pda::tc_gemm((const __nv_bfloat16 *)d_A, (const __nv_bfloat16 *)d_B, M, N, K, d_bias,
                                      epilogue, d_outF, (__nv_bfloat16 *)d_outB, d_preact, s);
  if (e == cudaSuccess) e = cudaStreamSynchronize(s);
  if (work) cudaFree(work);
  if (e != cudaSuccess) {
    pda::set_last_error(std::string("pda_tc_gemm_bf16: ") + cudaGetErrorString(e));
    return PDA_ERR_CUDA;
  }
  if (pda::tc_gemm_error_and_clear() != 0) {
    pda::set_last_error("pda_tc_gemm_bf16: a tensor-core wait timed out");
    return PDA_ERR_CUDA;
  }
  return PDA_OK;
}

}  // extern "C"
