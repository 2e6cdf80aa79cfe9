// Host interface of the tcgen05 BF16 GEMM (kernels in tc_gemm.cuh, launchers
// in mlp.cu).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace pda {
namespace tc {
enum Epilogue : int { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_ELU = 2 };

// byte offset of element (r, k) of a 64-column bf16 operand slice in the
// canonical K-major no-swizzle layout of tcgen05: 8 x 16-byte core matrices,
// the two adjacent in K 128 bytes apart, the 8-row groups 1024 bytes apart
__host__ __device__ inline uint32_t slice_offset(int r, int k) {
  return (uint32_t)((((r >> 3) << 3) + (k >> 3)) << 7) + (uint32_t)((r & 7) << 4) + (uint32_t)((k & 7) << 1);
}
// element index of (r, k) of a 16-row operand in the blocked layout of
// tc_gemm_thin_blocked's B: one 2 KB slice per 64 columns
__host__ __device__ inline long thin_b_index(int r, long k) {
  return ((k >> 6) * 2048 + (long)slice_offset(r, (int)(k & 63))) / 2;
}
}  // namespace tc

// C[M x N] = A[M x K] B[N x K]^T (+ bias, ELU); K a multiple of 64
cudaError_t tc_gemm(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K, const float *bias,
                    int epi, float *outF, __nv_bfloat16 *outB, float *preact, cudaStream_t s);
// same with split K when few output tiles would leave SMs idle (`work`:
// scratch of workFloats floats for the partial sums)
cudaError_t tc_gemm_splitk(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                           const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact, float *work,
                           long workFloats, cudaStream_t s);
// a row-major [M x K] bf16 operand in the blocked layout of
// tc_gemm_thin_blocked: rowsPerSlice = 128 for A ([tiles][K / 64] slices of
// 128 x 64, rows past M zero), 16 for B (M <= 16); K a multiple of 64
cudaError_t tc_block_operand(const __nv_bfloat16 *W, long M, long K, int rowsPerSlice, __nv_bfloat16 *Wb,
                             cudaStream_t s);
// partial[z][M][16] = the split-K partial sums of A B^T over `splits` slices
// of K, A and B in the blocked layout (one bulk copy per slice)
cudaError_t tc_gemm_thin_blocked(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long K, int splits,
                                 float *partial, cudaStream_t s);
// 1 if a GEMM gave up waiting on the tensor core since the last call (clears it)
int tc_gemm_error_and_clear();

}  // namespace pda
