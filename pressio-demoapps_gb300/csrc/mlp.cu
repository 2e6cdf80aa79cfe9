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

// lifts the dynamic shared-memory limit of one GEMM instantiation (once)
template <int BN_, int ST>
static cudaError_t gemm_attr() {
  static bool done = false;
  if (!done) {
    cudaError_t e = cudaFuncSetAttribute(tc::k_gemm_tn<BN_, ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::smem_bytes(BN_, ST));
    if (e != cudaSuccess) return e;
    done = true;
  }
  return cudaSuccess;
}

// one launch of k_gemm_tn (128 x 128 tiles, two stages) over all output
// tiles and `splits` K ranges of `per` slices
static cudaError_t launch_gemm(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                               const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact,
                               int splits, int per, float *partial, cudaStream_t s) {
  int *err = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void **)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const unsigned mt = (unsigned)((M + tc::BM - 1) / tc::BM);
  e = gemm_attr<tc::BN, tc::STAGES>();
  if (e != cudaSuccess) return e;
  tc::k_gemm_tn<tc::BN, tc::STAGES>
      <<<dim3((unsigned)((N + tc::BN - 1) / tc::BN), mt, (unsigned)splits), tc::THREADS, tc::SMEM_BYTES, s>>>(
          A, B, M, N, K, bias, epi, outF, outB, preact, err, per, partial);
  return cudaGetLastError();
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
  static int sms = 0;
  if (sms == 0) {
    int dev = 0;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    if (sms <= 0) sms = 1;
  }
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

cudaError_t tc_block_operand(const __nv_bfloat16 *W, long M, long K, int rowsPerSlice, __nv_bfloat16 *Wb,
                             cudaStream_t s) {
  if (K % tc::BK != 0 || (rowsPerSlice != tc::BM && !(rowsPerSlice == tc::THIN_BN && M <= tc::THIN_BN)))
    return cudaErrorInvalidValue;
  const long n = (M + rowsPerSlice - 1) / rowsPerSlice * (K / tc::BK) * rowsPerSlice * (tc::BK / 8);
  tc::k_block_operand<<<(unsigned)((n + 255) / 256), 256, 0, s>>>(W, M, K, rowsPerSlice, Wb);
  return cudaGetLastError();
}

cudaError_t tc_gemm_thin_blocked(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long K, int splits,
                                 float *partial, cudaStream_t s) {
  constexpr int ST = tc::THIN_STAGES;
  // the larger dynamic shared memory is a per-device function attribute
  constexpr int kMaxDev = 64;
  static bool attr[kMaxDev] = {};
  int dev = 0;
  cudaError_t ed = cudaGetDevice(&dev);
  if (ed != cudaSuccess) return ed;
  if (dev < 0 || dev >= kMaxDev || !attr[dev]) {
    cudaError_t e = cudaFuncSetAttribute(tc::k_gemm_thin_blocked<ST>, cudaFuncAttributeMaxDynamicSharedMemorySize,
                                         tc::blocked_smem_bytes(ST));
    if (e != cudaSuccess) return e;
    if (dev >= 0 && dev < kMaxDev) attr[dev] = true;
  }
  int *err = nullptr;
  cudaError_t e = cudaGetSymbolAddress((void **)&err, g_tc_err);
  if (e != cudaSuccess) return e;
  const int kt = (int)(K / tc::BK);
  splits = std::max(1, std::min(splits, kt));
  const int per = (kt + splits - 1) / splits;
  dim3 grid((unsigned)((M + tc::BM - 1) / tc::BM), (unsigned)splits);
  tc::k_gemm_thin_blocked<ST><<<grid, tc::THREADS, tc::blocked_smem_bytes(ST), s>>>(Ablk, Bblk, M, kt, per, partial,
                                                                                    err);
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
