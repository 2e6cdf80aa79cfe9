// Host interface of the tcgen05 BF16 GEMM (kernels in tc_gemm.cuh, launchers
// in mlp.cu).
#pragma once

#include <cstdint>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "adam.cuh"

namespace pda {
namespace tc {
enum Epilogue : int { EPI_NONE = 0, EPI_BIAS = 1, EPI_BIAS_ELU = 2 };

// Epilogue of a weight-gradient product C = dW [M x N]: the Adam update of
// the fp32 weights W (moments m, v) and the refresh of their bf16 copy Wb
// [M x N] and, when WbT is given, of its transpose [N x M].  Columns at or
// past `cols` are padding: W, m and v stay, both bf16 copies get 0.
struct AdamEpi {
  float *W = nullptr, *m = nullptr, *v = nullptr;
  __nv_bfloat16 *Wb = nullptr, *WbT = nullptr;
  long cols = 0;
  AdamCoef coef{};
  // bf16 copies in the blocked operand layout (Wb with N / 64 slices, WbT
  // with M / 64) instead of row-major
  bool blocked = false;
};
// Epilogue of the output layer's product in training: Y = C + bias is the
// reconstruction of X [M x N] (bf16); writes dY = bf16(gscale (Y - X)) as
// [M x N] and as its transpose dYT [N x M], and one double per CTA, the sum of
// (Y - X)^2 over its tile, to partial[blockIdx.y * gridDim.x + blockIdx.x].
struct MseEpi {
  const __nv_bfloat16 *X = nullptr;
  __nv_bfloat16 *dY = nullptr, *dYT = nullptr;
  float gscale = 0.f;
  double *partial = nullptr;
  // dY in the blocked operand layout with N / 64 slices instead of row-major
  bool blocked = false;
};
// Epilogue of the thin GEMM as the ROM decoder's output layer (one K split):
// row r of C = [c0, c1..cK] (the layer's output and its latent derivatives)
// becomes y[r] = uref[r] + scale[r] (c0 + b3[r]) and D[r][j] = scale[r] c(1+j).
struct ThinDecode {
  const float *b3 = nullptr;
  const double *uref = nullptr, *scale = nullptr;
  double *y = nullptr, *D = nullptr;
  int K = 0;  // latent columns, at most 15
};

// byte offset of element (r, k) of a 64-column bf16 operand slice in the
// canonical K-major no-swizzle layout of tcgen05: 8 x 16-byte core matrices,
// the two adjacent in K 128 bytes apart, the 8-row groups 1024 bytes apart
__host__ __device__ inline uint32_t slice_offset(int r, int k) {
  return (uint32_t)((((r >> 3) << 3) + (k >> 3)) << 7) + (uint32_t)((r & 7) << 4) + (uint32_t)((k & 7) << 1);
}
// element index of (r, k) of an operand of `kt` 64-column slices in the
// blocked layout of k_gemm_blocked: 128 x 64 blocks (16 KB) stored
// [r / 128][k / 64], each in the canonical layout of slice_offset
__host__ __device__ inline long blocked_index(long r, long k, long kt) {
  return ((((r >> 7) * kt) + (k >> 6)) << 13) + (long)(slice_offset((int)(r & 127), (int)(k & 63)) >> 1);
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
// C = A B^T is the gradient of a weight matrix [M x N]; the epilogue applies
// Adam to it (no split K; N a multiple of 4, M even, 16-byte aligned W, m, v)
cudaError_t tc_gemm_adam(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K,
                         const tc::AdamEpi &adam, cudaStream_t s);
// C = A B^T + bias is a reconstruction of X; the epilogue writes the squared
// error's gradient and per-CTA sums of squares (no split K; N a multiple of
// 16); `partial` holds ceil(M / 128) * ceil(N / 128) doubles
cudaError_t tc_gemm_mse(const __nv_bfloat16 *A, const __nv_bfloat16 *B, long M, long N, long K, const float *bias,
                        const tc::MseEpi &mse, cudaStream_t s);
// C = A B^T (+ bias, ELU) with both operands in the blocked layout
// (blocked_index; rows past M or N zero), one bulk copy per 16 KB slice, K
// split over CTAs into `work` when the output tiles are few; mse (optional)
// as in tc_gemm_mse
cudaError_t tc_gemm_blocked(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long N, long K,
                            const float *bias, int epi, float *outF, __nv_bfloat16 *outB, float *preact,
                            const tc::MseEpi *mse, float *work, long workFloats, cudaStream_t s);
// fp32 [R x C] -> bf16 in the blocked layout, as the operand [R x C]
// (trans = 0, C / 64 slices) or as its transpose [C x R] (trans = 1, R / 64
// slices); rows past the operand's end are left alone
cudaError_t tc_to_bf16_blocked(const float *W, long R, long C, int trans, __nv_bfloat16 *out, cudaStream_t s);
// a row-major [M x K] bf16 operand in the blocked layout of
// tc_gemm_thin_blocked: rowsPerSlice = 128 for A ([tiles][K / 64] slices of
// 128 x 64, rows past M zero), 16 for B (M <= 16); K a multiple of 64
cudaError_t tc_block_operand(const __nv_bfloat16 *W, long M, long K, int rowsPerSlice, __nv_bfloat16 *Wb,
                             cudaStream_t s);
// partial[z][M][16] = the split-K partial sums of A B^T over `splits` slices
// of K, A and B in the blocked layout (one bulk copy per slice)
cudaError_t tc_gemm_thin_blocked(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long K, int splits,
                                 float *partial, cudaStream_t s);
// sets the thin GEMM's shared-memory attribute on the current device (call
// before capturing a launch of it into a graph)
cudaError_t tc_gemm_thin_prepare();
// the same product over the whole K in one pass per row tile, finished in
// the epilogue as the decoder's output (ThinDecode)
cudaError_t tc_gemm_thin_decode(const __nv_bfloat16 *Ablk, const __nv_bfloat16 *Bblk, long M, long K,
                                const tc::ThinDecode &dec, cudaStream_t s);
// 1 if a GEMM gave up waiting on the tensor core since the last call (clears it)
int tc_gemm_error_and_clear();

}  // namespace pda
