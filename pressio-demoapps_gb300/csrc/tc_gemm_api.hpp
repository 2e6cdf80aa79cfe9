// Host interface of the tcgen05 BF16 GEMM (kernels in tc_gemm.cuh, launchers
// in mlp.cu).
#pragma once

#include <cuda_bf16.h>
#include <cuda_runtime.h>

namespace pda {
namespace tc {
enum Epilogue : int { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_ELU = 2 };
}  // namespace tc

// C[M x N] = A[M x K] B[N x K]^T (+ bias, ELU); K a multiple of 64
cudaError_t tc_gemm(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K, const float *bias,
                    int epi, float *outF, __nv_bfloat16 *outB, float *preact, cudaStream_t s);
// same with split K when few output tiles would leave SMs idle (`work`:
// scratch of workFloats floats for the partial sums)
cudaError_t tc_gemm_splitk(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                           const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact, float *work,
                           long workFloats, cudaStream_t s);
// the partial sums of A B^T over `splits` slices of K, partial[z][M][N] (raw
// fp32, no epilogue); the caller adds them in slice order
cudaError_t tc_gemm_partials(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K, int splits,
                             float *partial, cudaStream_t s);
// 1 if a GEMM gave up waiting on the tensor core since the last call (clears it)
int tc_gemm_error_and_clear();

}  // namespace pda
