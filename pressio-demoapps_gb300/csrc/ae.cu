// MLP autoencoder for the learned-manifold ROM, trained on the device.
//
//   encoder  n -> ha (ELU) -> hb (ELU) -> k          (k padded to 64 inside)
//   decoder  k -> hb (ELU) -> ha (ELU) -> n          (full-width output)
//
// Weights live as fp32 masters with Adam moments; every step refreshes bf16
// copies (and bf16 transposes where a backward GEMM needs W^T) that feed the
// tcgen05 GEMM (fp32 accumulation in tensor memory).  Activations are stored
// in bf16 for the next GEMM and in fp32 before the activation for the
// backward pass.  Loss: mean squared reconstruction error.
//
// One training step is a single pass over the weights: the output layer's
// GEMM epilogue forms the error gradient (and its transpose) without storing
// the reconstruction, and each weight-gradient GEMM's epilogue applies Adam
// to its tile and writes the refreshed bf16 copies, so the fp32 gradients of
// the weights never reach memory.
//
// Every product of the forward and backward pass is C = A B^T with both
// operands K-major:
//   forward   H_l   = act(H_{l-1} W_l^T + b_l)
//   backward  dW_l  = dA_l^T H_{l-1}       (A = dA_l^T, B = H_{l-1}^T)
//             dH_{l-1} = dA_l W_l          (B = W_l^T)
// so the transposes of dA_l, H_{l-1} and W_l are formed by a tiled kernel.
#include <algorithm>
#include <cmath>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include <cuda_bf16.h>
#include <cuda_runtime.h>

#include "problem_impl.hpp"
#include "tc_gemm_api.hpp"

namespace pda {

namespace ae {

using bf16 = __nv_bfloat16;

__device__ __forceinline__ uint64_t splitmix(uint64_t x) {
  x += 0x9E3779B97F4A7C15ull;
  x = (x ^ (x >> 30)) * 0xBF58476D1CE4E5B9ull;
  x = (x ^ (x >> 27)) * 0x94D049BB133111EBull;
  return x ^ (x >> 31);
}

// uniform(-a, a) in the first `cols` columns of each row, zero elsewhere
__global__ void k_init_uniform(float *w, long rows, long ld, long cols, float a, uint64_t seed) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= rows * ld) return;
  const long c = i % ld;
  if (c >= cols) {
    w[i] = 0.f;
    return;
  }
  const uint64_t r = splitmix(seed ^ (uint64_t)i * 0x2545F4914F6CDD1Dull);
  const float u = (float)((r >> 40) * (1.0 / 16777216.0));  // [0, 1)
  w[i] = (2.f * u - 1.f) * a;
}

__global__ void k_to_bf16(const float *__restrict__ x, bf16 *__restrict__ y, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] = __float2bfloat16_rn(x[i]);
}

// out[c][r] = in[r][c] for an R x C bf16 matrix (32 x 32 tiles)
__global__ void k_transpose(const bf16 *__restrict__ in, bf16 *__restrict__ out, long R, long C) {
  __shared__ bf16 t[32][33];
  const long c0 = (long)blockIdx.x * 32, r0 = (long)blockIdx.y * 32;
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const long r = r0 + j, c = c0 + threadIdx.x;
    if (r < R && c < C) t[j][threadIdx.x] = in[r * C + c];
  }
  __syncthreads();
  for (int j = threadIdx.y; j < 32; j += blockDim.y) {
    const long c = c0 + j, r = r0 + threadIdx.x;
    if (r < R && c < C) out[c * R + r] = t[threadIdx.x][j];
  }
}

// rows idx[i] of the dataset (bf16 [ns x n]) -> X batch
__global__ void k_gather_rows(const bf16 *__restrict__ data, const int64_t *__restrict__ idx, long n, long rows,
                              bf16 *__restrict__ X) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;  // in 8-element chunks
  const long chunks = n / 8;
  if (i >= rows * chunks) return;
  const long r = i / chunks, c = i % chunks;
  reinterpret_cast<uint4 *>(X + r * n)[c] = reinterpret_cast<const uint4 *>(data + idx[r] * n)[c];
}

// dA = dH * elu'(pre) -> bf16 (pre is the value before the ELU)
__global__ void k_elu_back(const float *__restrict__ dH, const float *__restrict__ pre, bf16 *__restrict__ dA,
                           long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const float a = pre[i];
  dA[i] = __float2bfloat16_rn(dH[i] * (a > 0.f ? 1.f : expf(a)));
}

// column sums of a bf16 [rows x cols] matrix (bias gradients), fixed order;
// with `b` given, also the Adam update of the bias b (moments mb, vb) on the
// first `realCols` entries
__global__ void k_colsum(const bf16 *__restrict__ d, long rows, long cols, float *__restrict__ out,
                         float *__restrict__ b, float *__restrict__ mb, float *__restrict__ vb, long realCols,
                         AdamCoef coef) {
  const long c = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (c >= cols) return;
  float s = 0.f;
  for (long r = 0; r < rows; ++r) s += __bfloat162float(d[r * cols + c]);
  out[c] = s;
  if (b && c < realCols) b[c] = adam_update(b[c], mb[c], vb[c], s, coef);
}

// row sums of a bf16 [rows x cols] matrix, one warp per row (lane l adds
// columns l, l + 32, ... in order, then a fixed butterfly over the lanes):
// the bias gradient from a transposed error gradient; Adam on b as in
// k_colsum.  Launch rows * 32 threads.
__global__ void k_rowsum(const bf16 *__restrict__ d, long rows, long cols, float *__restrict__ out,
                         float *__restrict__ b, float *__restrict__ mb, float *__restrict__ vb, long realRows,
                         AdamCoef coef) {
  const long r = ((long)blockIdx.x * blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31;
  if (r >= rows) return;  // whole warps
  float s = 0.f;
  for (long c = lane; c < cols; c += 32) s += __bfloat162float(d[r * cols + c]);
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if (lane == 0) {
    out[r] = s;
    if (b && r < realRows) b[r] = adam_update(b[r], mb[r], vb[r], s, coef);
  }
}

// Adam on a [n / ld x ld] parameter block with gradient g, refreshing the
// bf16 copy wb when given; entries outside the first `cols` columns of each
// row (latent padding) stay 0.
__global__ void k_adam(float *__restrict__ w, float *__restrict__ m, float *__restrict__ v,
                       const float *__restrict__ g, bf16 *__restrict__ wb, long n, long ld, long cols, AdamCoef coef) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (i % ld >= cols) {
    if (wb) wb[i] = __float2bfloat16_rn(0.f);
    return;
  }
  float mi = m[i], vi = v[i];
  const float wi = adam_update(w[i], mi, vi, g[i], coef);
  m[i] = mi;
  v[i] = vi;
  w[i] = wi;
  if (wb) wb[i] = __float2bfloat16_rn(wi);
}

// ---------------------------------------------------------------- layers
template <class T> struct Buf {
  T *p = nullptr;
  size_t n = 0;
  Buf() = default;
  Buf(const Buf &) = delete;
  Buf &operator=(const Buf &) = delete;
  ~Buf() {
    if (p) cudaFree(p);
  }
  void alloc(size_t c) {
    if (p && n >= c) return;
    if (p) cudaFree(p);
    p = nullptr;
    n = 0;
    if (cudaMalloc((void **)&p, std::max<size_t>(c, 1) * sizeof(T)) != cudaSuccess)
      throw Error(PDA_ERR_OUT_OF_MEMORY, "autoencoder: device allocation failed");
    n = c;
  }
};

struct Layer {
  long in = 0, out = 0;      // padded sizes (multiples of 64 where they are GEMM K)
  long inReal = 0, outReal = 0;
  bool elu = false;
  Buf<float> W, b, mW, vW, mb, vb, gW, gb;
  Buf<bf16> Wb, WbT;  // [out x in], [in x out]: row-major, or blocked operands
  bool needT = false;
  // the wide layers (first and last) keep their bf16 copies in the blocked
  // operand layout for the bulk-copy GEMM (their forward and input-gradient
  // products have K = n or N = n)
  bool blk = false;
};

}  // namespace ae
}  // namespace pda

struct pda_ae {
  long n = 0;
  int k = 0, kp = 0, ha = 0, hb = 0;
  cudaStream_t s = nullptr;
  pda::ae::Layer L[6];
  int batch = 0;
  // activations for one batch
  pda::ae::Buf<pda::ae::bf16> X, XT, Hb[6], HbT[6], dA, dAT;
  // blocked operands of the wide layers' GEMMs: the batch, layer 4's output,
  // the output error gradient (rows padded to 128 and zero)
  pda::ae::Buf<pda::ae::bf16> Xblk, H4blk, dYblk;
  pda::ae::Buf<float> pre[6], Y, dH;
  pda::ae::Buf<float> work;
  pda::ae::Buf<double> lossPart;
  pda::ae::Buf<int64_t> idx;
  long workFloats = 0;
  int64_t step = 0;
  // Adam fused into the weight-gradient GEMMs' epilogues (false: the
  // gradients are stored and a separate optimizer pass follows)
  bool fusedAdam = true;
};

namespace pda {
namespace ae {
namespace {

inline unsigned g1(long n, int b = 256) { return (unsigned)((n + b - 1) / b); }

void check(cudaError_t e, const char *what) {
  if (e != cudaSuccess) throw Error(PDA_ERR_CUDA, std::string(what) + ": " + cudaGetErrorString(e));
}

void transpose(const bf16 *in, bf16 *out, long R, long C, cudaStream_t s) {
  dim3 grid((unsigned)((C + 31) / 32), (unsigned)((R + 31) / 32));
  k_transpose<<<grid, dim3(32, 8), 0, s>>>(in, out, R, C);
}

void refresh_bf16(Layer &l, cudaStream_t s) {
  if (l.blk) {
    check(tc_to_bf16_blocked(l.W.p, l.out, l.in, 0, l.Wb.p, s), "bf16 blocked copy");
    if (l.needT) check(tc_to_bf16_blocked(l.W.p, l.out, l.in, 1, l.WbT.p, s), "bf16 blocked transpose");
    return;
  }
  k_to_bf16<<<g1(l.out * l.in), 256, 0, s>>>(l.W.p, l.Wb.p, l.out * l.in);
  if (l.needT) transpose(l.Wb.p, l.WbT.p, l.out, l.in, s);
}

inline long pad128(long r) { return (r + 127) / 128 * 128; }

void alloc_zero(Buf<bf16> &b, size_t n, cudaStream_t s) {
  b.alloc(n);
  check(cudaMemsetAsync(b.p, 0, n * sizeof(bf16), s), "memset");
}

void ensure_batch(pda_ae &A, int B) {
  if (A.batch >= B) return;
  A.batch = B;
  const long n = A.n;
  A.X.alloc((size_t)B * n);
  A.XT.alloc((size_t)B * n);
  for (int l = 0; l < 6; ++l) {
    A.Hb[l].alloc((size_t)B * A.L[l].out);
    A.HbT[l].alloc((size_t)B * A.L[l].out);
    A.pre[l].alloc((size_t)B * A.L[l].out);
  }
  A.Y.alloc((size_t)B * n);
  alloc_zero(A.Xblk, (size_t)pad128(B) * n, A.s);
  alloc_zero(A.H4blk, (size_t)pad128(B) * A.L[4].out, A.s);
  alloc_zero(A.dYblk, (size_t)pad128(B) * n, A.s);
  long maxOut = 0;
  for (auto &l : A.L) maxOut = std::max(maxOut, std::max(l.out, l.in));
  A.dA.alloc((size_t)B * std::max(maxOut, n));
  A.dAT.alloc((size_t)B * std::max(maxOut, n));
  A.dH.alloc((size_t)B * maxOut);
  A.workFloats = 64L * B * std::max<long>(A.ha, 1024);
  A.work.alloc((size_t)A.workFloats);
  A.lossPart.alloc((size_t)std::max<long>(1024, ((n + 127) / 128) * ((B + 127) / 128)));
  A.idx.alloc((size_t)B);
}

void gemm(pda_ae &A, const bf16 *a, const bf16 *b, long M, long N, long K, const float *bias, int epi, float *outF,
          bf16 *outB, float *pre) {
  check(tc_gemm_splitk(a, b, M, N, K, bias, epi, outF, outB, pre, A.work.p, A.workFloats, A.s), "tc gemm");
}

// forward of a batch already in A.X: fills Hb / pre; the output layer either
// writes Y (train = false) or, in training, the reconstruction error's
// gradient dY (blocked in A.dYblk, and its transpose in A.dAT) and per-CTA
// sums of squares (A.lossPart, `parts` of them) without storing Y
void forward(pda_ae &A, int B, bool train, long *parts = nullptr) {
  const bf16 *in = A.X.p;
  for (int l = 0; l < 6; ++l) {
    Layer &ly = A.L[l];
    if (l == 0) {
      // K = n: both operands blocked, K split over the SMs
      check(tc_block_operand(A.X.p, B, A.n, 128, A.Xblk.p, A.s), "block X");
      check(tc_gemm_blocked(A.Xblk.p, ly.Wb.p, B, ly.out, ly.in, ly.b.p, tc::EPI_BIAS_ELU, nullptr, A.Hb[0].p,
                            A.pre[0].p, nullptr, A.work.p, A.workFloats, A.s),
            "tc gemm (first layer)");
      in = A.Hb[0].p;
    } else if (l == 5) {
      // N = n: layer 4's output blocked against the blocked weights
      check(tc_block_operand(in, B, ly.in, 128, A.H4blk.p, A.s), "block H4");
      if (train) {
        tc::MseEpi me;
        me.X = A.X.p;
        me.dY = A.dYblk.p;
        me.blocked = true;
        me.dYT = A.dAT.p;
        me.gscale = 2.f / (float)((long)B * A.n);
        me.partial = A.lossPart.p;
        check(tc_gemm_blocked(A.H4blk.p, ly.Wb.p, B, ly.out, ly.in, ly.b.p, tc::EPI_BIAS, nullptr, nullptr, nullptr,
                              &me, nullptr, 0, A.s),
              "tc gemm (output layer, squared error)");
        if (parts) *parts = ((ly.out + 127) / 128) * ((B + 127) / 128);  // one per 128 x 128 output tile
      } else {
        check(tc_gemm_blocked(A.H4blk.p, ly.Wb.p, B, ly.out, ly.in, ly.b.p, tc::EPI_BIAS, A.Y.p, nullptr, nullptr,
                              nullptr, nullptr, 0, A.s),
              "tc gemm (output layer)");
      }
    } else {
      gemm(A, in, ly.Wb.p, B, ly.out, ly.in, ly.b.p, ly.elu ? tc::EPI_BIAS_ELU : tc::EPI_BIAS, nullptr, A.Hb[l].p,
           A.pre[l].p);
      in = A.Hb[l].p;
    }
  }
}


// gradients of the mean squared error of the batch in A.X; returns the loss
// (sum of squares / (B n)) on the host.  With `coef`, each layer's weights
// and bias take their Adam step as soon as their gradients exist (fused into
// the weight-gradient GEMM and the bias column sums); the layer's input
// gradient is formed first, from the weights before the step.
double forward_backward(pda_ae &A, int B, const AdamCoef *coef) {
  long parts = 0;
  forward(A, B, true, &parts);
  // layer 5 (output): dA5 = dY (blocked), its transpose already in A.dAT
  const bf16 *dAcur = A.dYblk.p;
  for (int l = 5; l >= 0; --l) {
    Layer &ly = A.L[l];
    const bf16 *hin = l == 0 ? A.X.p : A.Hb[l - 1].p;
    const long inW = ly.in, outW = ly.out;
    if (l < 5) transpose(dAcur, A.dAT.p, B, outW, A.s);
    bf16 *hinT = (l == 0) ? A.XT.p : A.HbT[l - 1].p;
    transpose(hin, hinT, B, inW, A.s);
    const AdamCoef c0{};
    if (l == 5)  // bias gradient from the transposed error gradient [n x B]
      k_rowsum<<<g1(outW * 32), 256, 0, A.s>>>(A.dAT.p, outW, B, ly.gb.p, coef ? ly.b.p : nullptr, ly.mb.p,
                                               ly.vb.p, ly.outReal, coef ? *coef : c0);
    else
      k_colsum<<<g1(outW), 256, 0, A.s>>>(dAcur, B, outW, ly.gb.p, coef ? ly.b.p : nullptr, ly.mb.p, ly.vb.p,
                                          ly.outReal, coef ? *coef : c0);
    // dH_in = dA W: B operand = W^T [in x out]
    if (l == 5)
      check(tc_gemm_blocked(A.dYblk.p, ly.WbT.p, B, inW, outW, nullptr, tc::EPI_NONE, A.dH.p, nullptr, nullptr,
                            nullptr, A.work.p, A.workFloats, A.s),
            "tc gemm (output layer, input gradient)");
    else if (l > 0)
      gemm(A, dAcur, ly.WbT.p, B, inW, outW, nullptr, tc::EPI_NONE, A.dH.p, nullptr, nullptr);
    // dW = dA^T H_in: A = dA^T [out x B], B = H_in^T [in x B]
    if (coef) {
      tc::AdamEpi ad;
      ad.W = ly.W.p;
      ad.m = ly.mW.p;
      ad.v = ly.vW.p;
      ad.Wb = ly.Wb.p;
      ad.WbT = ly.needT ? ly.WbT.p : nullptr;
      ad.cols = ly.inReal;
      ad.coef = *coef;
      ad.blocked = ly.blk;
      check(tc_gemm_adam(A.dAT.p, hinT, outW, inW, B, ad, A.s), "tc gemm (weight gradient, Adam)");
    } else {
      gemm(A, A.dAT.p, hinT, outW, inW, B, nullptr, tc::EPI_NONE, ly.gW.p, nullptr, nullptr);
    }
    if (l == 0) break;
    Layer &prev = A.L[l - 1];
    // dA of the layer below overwrites A.dA only after its last use above
    if (prev.elu) {
      k_elu_back<<<g1((long)B * inW), 256, 0, A.s>>>(A.dH.p, A.pre[l - 1].p, A.dA.p, (long)B * inW);
    } else {
      k_to_bf16<<<g1((long)B * inW), 256, 0, A.s>>>(A.dH.p, A.dA.p, (long)B * inW);
    }
    dAcur = A.dA.p;
  }
  std::vector<double> h((size_t)parts);
  check(cudaMemcpyAsync(h.data(), A.lossPart.p, parts * sizeof(double), cudaMemcpyDeviceToHost, A.s), "loss copy");
  check(cudaStreamSynchronize(A.s), "sync");
  double sum = 0.;
  for (double v : h) sum += v;
  return sum / ((double)B * A.n);
}

// the optimizer pass over stored gradients (the unfused schedule)
void adam_step(pda_ae &A, const AdamCoef &coef) {
  for (auto &ly : A.L) {
    const long nw = ly.out * ly.in;
    k_adam<<<g1(nw), 256, 0, A.s>>>(ly.W.p, ly.mW.p, ly.vW.p, ly.gW.p, ly.blk ? nullptr : ly.Wb.p, nw, ly.in,
                                    ly.inReal, coef);
    k_adam<<<g1(ly.out), 256, 0, A.s>>>(ly.b.p, ly.mb.p, ly.vb.p, ly.gb.p, nullptr, ly.out, ly.out, ly.outReal,
                                        coef);
    if (ly.blk) {
      refresh_bf16(ly, A.s);
    } else if (ly.needT) {
      transpose(ly.Wb.p, ly.WbT.p, ly.out, ly.in, A.s);
    }
  }
}

void create(pda_ae &A, long n, int k, int ha, int hb, uint64_t seed, void *stream) {
  PDA_REQUIRE(n > 0 && n % 64 == 0, PDA_ERR_INVALID_ARGUMENT, "autoencoder: n must be a positive multiple of 64");
  PDA_REQUIRE(k >= 1 && k <= 64, PDA_ERR_INVALID_ARGUMENT, "autoencoder: latent size must be in [1, 64]");
  PDA_REQUIRE(ha > 0 && ha % 64 == 0 && hb > 0 && hb % 64 == 0, PDA_ERR_INVALID_ARGUMENT,
              "autoencoder: hidden widths must be positive multiples of 64");
  A.n = n;
  A.k = k;
  A.kp = 64;
  A.ha = ha;
  A.hb = hb;
  A.s = (cudaStream_t)stream;
  const long ins[6] = {n, ha, hb, 64, hb, ha};
  const long outs[6] = {ha, hb, 64, hb, ha, n};
  const long insR[6] = {n, ha, hb, k, hb, ha};
  const long outsR[6] = {ha, hb, k, hb, ha, n};
  const bool elus[6] = {true, true, false, true, true, false};
  for (int l = 0; l < 6; ++l) {
    Layer &ly = A.L[l];
    ly.in = ins[l];
    ly.out = outs[l];
    ly.inReal = insR[l];
    ly.outReal = outsR[l];
    ly.elu = elus[l];
    ly.needT = l > 0;  // dH_in of layer 0 (the data) is never needed
    ly.blk = l == 0 || l == 5;
    const long nw = ly.out * ly.in;
    ly.W.alloc(nw);
    ly.mW.alloc(nw);
    ly.vW.alloc(nw);
    ly.gW.alloc(nw);
    ly.b.alloc(ly.out);
    ly.mb.alloc(ly.out);
    ly.vb.alloc(ly.out);
    ly.gb.alloc(ly.out);
    if (ly.blk) {  // blocked operands: rows padded to 128 and zero
      alloc_zero(ly.Wb, (size_t)pad128(ly.out) * ly.in, A.s);
      if (ly.needT) alloc_zero(ly.WbT, (size_t)pad128(ly.in) * ly.out, A.s);
    } else {
      ly.Wb.alloc(nw);
      if (ly.needT) ly.WbT.alloc(nw);
    }
    // Glorot uniform on the real fan-in / fan-out; padding rows / columns 0
    const float a = std::sqrt(6.f / (float)(ly.inReal + ly.outReal));
    k_init_uniform<<<g1(nw), 256, 0, A.s>>>(ly.W.p, ly.out, ly.in, ly.inReal, a, seed + 7919ull * (l + 1));
    if (ly.outReal < ly.out)  // latent padding rows of the encoder's last layer
      check(cudaMemsetAsync(ly.W.p + ly.outReal * ly.in, 0, (ly.out - ly.outReal) * ly.in * sizeof(float), A.s),
            "memset");
    for (auto *bb : {&ly.b, &ly.mb, &ly.vb, &ly.mW, &ly.vW})
      check(cudaMemsetAsync(bb->p, 0, bb->n * sizeof(float), A.s), "memset");
    refresh_bf16(ly, A.s);
  }
  check(cudaStreamSynchronize(A.s), "init");
}

}  // namespace
}  // namespace ae
}  // namespace pda

using pda::Error;

extern "C" {

pda_status pda_ae_create(int64_t n, int latent, int ha, int hb, uint64_t seed, void *stream, pda_ae **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(out, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_ptr<pda_ae> A(new pda_ae);
  pda::ae::create(*A, n, latent, ha, hb, seed, stream);
  *out = A.release();
  PDA_API_END
}

void pda_ae_free(pda_ae *a) { delete a; }

pda_status pda_ae_train(pda_ae *A, const void *d_data, int64_t ns, int batch, int epochs, double lr, uint64_t seed,
                        double *losses) {
  PDA_API_BEGIN
  PDA_REQUIRE(A && d_data && ns > 0 && epochs >= 0, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  PDA_REQUIRE(batch > 0 && batch % 64 == 0 && batch <= ns, PDA_ERR_INVALID_ARGUMENT,
              "batch must be a positive multiple of 64, at most the number of snapshots");
  pda::ae::ensure_batch(*A, batch);
  const auto *data = (const pda::ae::bf16 *)d_data;
  std::vector<int64_t> perm((size_t)ns);
  uint64_t st = seed * 0x9E3779B97F4A7C15ull + 1;
  auto rnd = [&]() {
    st ^= st << 13;
    st ^= st >> 7;
    st ^= st << 17;
    return st;
  };
  for (int e = 0; e < epochs; ++e) {
    for (int64_t i = 0; i < ns; ++i) perm[(size_t)i] = i;
    for (int64_t i = ns - 1; i > 0; --i) std::swap(perm[(size_t)i], perm[(size_t)(rnd() % (uint64_t)(i + 1))]);
    double acc = 0.;
    int nbat = 0;
    for (int64_t b0 = 0; b0 + batch <= ns; b0 += batch) {
      PDA_CUDA(cudaMemcpyAsync(A->idx.p, perm.data() + b0, batch * sizeof(int64_t), cudaMemcpyHostToDevice, A->s));
      pda::ae::k_gather_rows<<<pda::ae::g1((long)batch * (A->n / 8)), 256, 0, A->s>>>(data, A->idx.p, A->n, batch,
                                                                                       A->X.p);
      A->step += 1;
      const pda::AdamCoef coef = pda::adam_coef((float)lr, (long)A->step);
      if (A->fusedAdam) {
        acc += pda::ae::forward_backward(*A, batch, &coef);
      } else {
        acc += pda::ae::forward_backward(*A, batch, nullptr);
        pda::ae::adam_step(*A, coef);
      }
      ++nbat;
    }
    if (losses) losses[e] = acc / std::max(nbat, 1);
  }
  PDA_CUDA(cudaStreamSynchronize(A->s));
  PDA_REQUIRE(pda::tc_gemm_error_and_clear() == 0, PDA_ERR_CUDA, "autoencoder: a tensor-core wait timed out");
  PDA_API_END
}

pda_status pda_ae_set_fused(pda_ae *A, int fused) {
  PDA_API_BEGIN
  PDA_REQUIRE(A, PDA_ERR_INVALID_ARGUMENT, "null argument");
  A->fusedAdam = fused != 0;
  PDA_API_END
}

pda_status pda_ae_reconstruct(pda_ae *A, const void *d_X, int64_t rows, float *d_Y, float *d_Z) {
  PDA_API_BEGIN
  PDA_REQUIRE(A && d_X && d_Y && rows > 0, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  const int B = 64;
  pda::ae::ensure_batch(*A, std::max(A->batch, B));
  for (int64_t r0 = 0; r0 < rows; r0 += B) {
    const long nr = std::min<int64_t>(B, rows - r0);
    PDA_CUDA(cudaMemsetAsync(A->X.p, 0, (size_t)B * A->n * sizeof(pda::ae::bf16), A->s));
    PDA_CUDA(cudaMemcpyAsync(A->X.p, (const pda::ae::bf16 *)d_X + r0 * A->n, nr * A->n * sizeof(pda::ae::bf16),
                             cudaMemcpyDeviceToDevice, A->s));
    pda::ae::forward(*A, B, false);
    PDA_CUDA(cudaMemcpyAsync(d_Y + r0 * A->n, A->Y.p, nr * A->n * sizeof(float), cudaMemcpyDeviceToDevice, A->s));
    if (d_Z) {
      // latent = layer 2 output (pre-activation, linear layer), first k columns
      PDA_CUDA(cudaMemcpy2DAsync(d_Z + r0 * A->k, A->k * sizeof(float), A->pre[2].p, 64 * sizeof(float),
                                 A->k * sizeof(float), nr, cudaMemcpyDeviceToDevice, A->s));
    }
  }
  PDA_CUDA(cudaStreamSynchronize(A->s));
  PDA_REQUIRE(pda::tc_gemm_error_and_clear() == 0, PDA_ERR_CUDA, "autoencoder: a tensor-core wait timed out");
  PDA_API_END
}

// loss and parameter gradients of one batch without an update (gradient
// checks); grads: concatenation over layers of [W (out x in, padded), b (out)]
pda_status pda_ae_gradients(pda_ae *A, const void *d_X, int batch, double *loss, float *d_grads) {
  PDA_API_BEGIN
  PDA_REQUIRE(A && d_X && batch > 0 && batch % 64 == 0, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  pda::ae::ensure_batch(*A, batch);
  PDA_CUDA(cudaMemcpyAsync(A->X.p, d_X, (size_t)batch * A->n * sizeof(pda::ae::bf16), cudaMemcpyDeviceToDevice, A->s));
  const double l = pda::ae::forward_backward(*A, batch, nullptr);
  if (loss) *loss = l;
  if (d_grads) {
    size_t off = 0;
    for (auto &ly : A->L) {
      const size_t nw = (size_t)ly.out * ly.in;
      PDA_CUDA(cudaMemcpyAsync(d_grads + off, ly.gW.p, nw * sizeof(float), cudaMemcpyDeviceToDevice, A->s));
      off += nw;
      PDA_CUDA(cudaMemcpyAsync(d_grads + off, ly.gb.p, ly.out * sizeof(float), cudaMemcpyDeviceToDevice, A->s));
      off += (size_t)ly.out;
    }
  }
  PDA_CUDA(cudaStreamSynchronize(A->s));
  PDA_REQUIRE(pda::tc_gemm_error_and_clear() == 0, PDA_ERR_CUDA, "autoencoder: a tensor-core wait timed out");
  PDA_API_END
}

// fp32 master weights of layer l (0..5), padded shapes: W [out x in], b [out]
pda_status pda_ae_layer(pda_ae *A, int l, float *d_W, float *d_b, int64_t *out_in) {
  PDA_API_BEGIN
  PDA_REQUIRE(A && l >= 0 && l < 6, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  auto &ly = A->L[l];
  if (out_in) {
    out_in[0] = ly.out;
    out_in[1] = ly.in;
  }
  if (d_W) PDA_CUDA(cudaMemcpy(d_W, ly.W.p, (size_t)ly.out * ly.in * sizeof(float), cudaMemcpyDeviceToDevice));
  if (d_b) PDA_CUDA(cudaMemcpy(d_b, ly.b.p, (size_t)ly.out * sizeof(float), cudaMemcpyDeviceToDevice));
  PDA_API_END
}

// overwrite the fp32 master weights of layer l (padded shapes) and refresh
// the bf16 copies (tests, warm starts)
pda_status pda_ae_set_layer(pda_ae *A, int l, const float *d_W, const float *d_b) {
  PDA_API_BEGIN
  PDA_REQUIRE(A && l >= 0 && l < 6 && d_W && d_b, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  auto &ly = A->L[l];
  PDA_CUDA(cudaMemcpy(ly.W.p, d_W, (size_t)ly.out * ly.in * sizeof(float), cudaMemcpyDeviceToDevice));
  PDA_CUDA(cudaMemcpy(ly.b.p, d_b, (size_t)ly.out * sizeof(float), cudaMemcpyDeviceToDevice));
  pda::ae::refresh_bf16(ly, A->s);
  PDA_CUDA(cudaStreamSynchronize(A->s));
  PDA_API_END
}

}  // extern "C"
