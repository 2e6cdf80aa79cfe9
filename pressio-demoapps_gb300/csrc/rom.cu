// Hyper-reduced LSPG (BDF1 / BDF2, Gauss-Newton with FP64 normal equations) on the
// device, over a sample-mesh problem, with an affine trial space
// (y = u_ref + Phi x) or a nonlinear manifold given by an MLP decoder
// (y = u_ref + scale * dec(x), dec = W3 elu(W2 elu(W1 x + b1) + b2) + b3
// evaluated only at the stencil-mesh rows).
//
// Per time step n -> n+1 and Gauss-Newton iteration (Pressio's
// LspgUnsteadyResidualJacobianPolicyHypRed, lspg_unsteady_rj_policy_hypred.hpp:
// 180-264, with the constants of ode_constants.hpp:57-73: BDF1 c_n = -1,
// c_f = -1; BDF2 c_n = -4/3, c_n-1 = 1/3, c_f = -2/3, its first step BDF1):
//   y      = trial state at the current latent x (stencil rows), D = dy/dx
//   V, Jf  = sample-mesh velocity and Jacobian at y (the library's kernels)
//   R      = cf V + (y + c_n y_n [+ c_n-1 y_n-1])|sample     cf = c_f dt
//   JR     = cf (Jf D) + D|sample
//   (JR^T JR) dx = JR^T R,  x <- x - dx               (FP64, Cholesky)
// Each kernel reads a per-step "converged" flag and returns at once after the
// correction fell below the tolerance, so a fixed number of iterations can be
// captured in one CUDA graph per step.
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
namespace rom {

constexpr int KMAX = 32;        // latent dimension limit

using Flags = LspgFlags;

// ------------------------------------------------------------ trial spaces
template <int K>
__global__ void k_decode_affine(long nst, const double *__restrict__ uref, const double *__restrict__ phi,
                                const double *__restrict__ x, double *__restrict__ y, int first, const Flags *f) {
  if (!first && f->converged) return;
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= nst) return;
  double acc = 0.;
#pragma unroll
  for (int c = 0; c < K; ++c) acc += phi[i * K + c] * x[c];
  y[i] = uref[i] + acc;
}

// bf16 copy of fp32 values that must already be bf16 values; *bad = 1 otherwise
__global__ void k_to_bf16_exact(const float *__restrict__ in, __nv_bfloat16 *__restrict__ out, long n,
                                int *__restrict__ bad) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const __nv_bfloat16 b = __float2bfloat16_rn(in[i]);
  out[i] = b;
  if (__bfloat162float(b) != in[i]) *bad = 1;
}

__device__ __forceinline__ float elu_f(float a) { return a > 0.f ? a : expm1f(a); }
__device__ __forceinline__ float delu_f(float a) { return a > 0.f ? 1.f : expf(a); }

// hidden layers: every block recomputes layer 1 (h1 x k, tiny) in shared
// memory, then layer 2 for its rows, one warp per row: h2[r] and
// T2[r][c] = elu'(a2_r) (W2 T1)_rc with T1 = diag(elu'(a1)) W1.  The lanes
// split the layer-1 width (coalesced reads of W2's row r), their 1 + k partial
// sums are added by a butterfly of shuffles.  Output Z[r][0] = h2,
// Z[r][1 + c] = T2 (fp32), and when Zb is given the same values as bf16 rows
// [1 + k (padded to 16)][h2] for the tensor-core output layer (its B operand,
// in the blocked slice layout of tc_gemm_thin_blocked).
constexpr int kHiddenWarps = 8;

template <int K, int H1>
__global__ void __launch_bounds__(kHiddenWarps * 32)
k_decode_hidden(int h2, const float *__restrict__ W1, const float *__restrict__ b1, const float *__restrict__ W2,
                const float *__restrict__ b2, const double *__restrict__ x, float *__restrict__ Z,
                __nv_bfloat16 *__restrict__ Zb, int first, const Flags *f) {
  if (!first && f->converged) return;
  static_assert(H1 % 32 == 0, "layer-1 width a multiple of the warp");
  constexpr int ld = 1 + K;
  __shared__ float sh1[H1];
  __shared__ float sT1[H1][K + 1];  // odd row length: lanes j, j+1 hit different banks
  __shared__ float sx[K];
  if (threadIdx.x < K) sx[threadIdx.x] = (float)x[threadIdx.x];
  __syncthreads();
  for (int r = threadIdx.x; r < H1; r += blockDim.x) {
    float a = b1[r];
#pragma unroll
    for (int c = 0; c < K; ++c) a += W1[r * K + c] * sx[c];
    sh1[r] = elu_f(a);
    const float d = delu_f(a);
#pragma unroll
    for (int c = 0; c < K; ++c) sT1[r][c] = d * W1[r * K + c];
  }
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const int r = blockIdx.x * kHiddenWarps + (threadIdx.x >> 5);
  if (r >= h2) return;
  const float *__restrict__ w = W2 + (long)r * H1;
  float wv[H1 / 32];
#pragma unroll
  for (int i = 0; i < H1 / 32; ++i) wv[i] = __ldg(w + lane + 32 * i);  // all loads in flight together
  float acc[ld];
#pragma unroll
  for (int c = 0; c < ld; ++c) acc[c] = 0.f;
#pragma unroll
  for (int i = 0; i < H1 / 32; ++i) {
    const int j = lane + 32 * i;
    acc[0] += wv[i] * sh1[j];
#pragma unroll
    for (int c = 0; c < K; ++c) acc[1 + c] += wv[i] * sT1[j][c];
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1)
#pragma unroll
    for (int c = 0; c < ld; ++c) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
  if (lane != 0) return;
  const float a = b2[r] + acc[0];
  const float d = delu_f(a);
  const float h = elu_f(a);
  Z[(long)r * ld] = h;
#pragma unroll
  for (int c = 0; c < K; ++c) Z[(long)r * ld + 1 + c] = d * acc[1 + c];
  if (Zb) {  // B operand of the output layer, blocked as tc_gemm_thin_blocked reads it
    Zb[tc::thin_b_index(0, r)] = __float2bfloat16_rn(h);
#pragma unroll
    for (int c = 0; c < K; ++c) Zb[tc::thin_b_index(1 + c, r)] = __float2bfloat16_rn(d * acc[1 + c]);
  }
}

// tensor-core output layer: [y-part | D-part] [nst x 16] = W3b [nst x h2]
// Zb^T (fp32), both operands in the blocked slice layout (one bulk copy per
// 64-column slice), finished in the GEMM's epilogue: y = uref + scale (C[., 0]
// + b3), D = scale C[., 1..k] (tc_gemm_thin_decode).

// output layer at the stencil rows: one warp per row (lanes over the hidden
// width, 8 weights in flight per lane), the [h2 | T2] block staged in shared
// memory by every block (h2 x (1+k) floats)
template <int K>
__global__ void __launch_bounds__(256)
k_decode_out(int h2, long nst, const float *__restrict__ W3, const float *__restrict__ b3,
             const double *__restrict__ uref, const double *__restrict__ scale, const float *__restrict__ Z,
             double *__restrict__ y, double *__restrict__ D, int first, const Flags *f) {
  if (!first && f->converged) return;
  extern __shared__ float sZ[];
  constexpr int ld = 1 + K;
  for (int i = threadIdx.x; i < h2 * ld; i += blockDim.x) sZ[i] = Z[i];
  __syncthreads();
  const int lane = threadIdx.x & 31;
  const long warps = (long)gridDim.x * (blockDim.x >> 5);
  for (long row = (long)blockIdx.x * (blockDim.x >> 5) + (threadIdx.x >> 5); row < nst; row += warps) {
    float acc[ld];
#pragma unroll
    for (int c = 0; c < ld; ++c) acc[c] = 0.f;
    const float *w = W3 + row * h2;
    int j = lane;
    for (; j + 32 * 7 < h2; j += 32 * 8) {
      float wv[8];
#pragma unroll
      for (int u = 0; u < 8; ++u) wv[u] = __ldg(w + j + 32 * u);
#pragma unroll
      for (int u = 0; u < 8; ++u) {
        const float *z = sZ + (j + 32 * u) * ld;
#pragma unroll
        for (int c = 0; c < ld; ++c) acc[c] += wv[u] * z[c];
      }
    }
    for (; j < h2; j += 32) {
      const float wj = __ldg(w + j);
      const float *z = sZ + j * ld;
#pragma unroll
      for (int c = 0; c < ld; ++c) acc[c] += wj * z[c];
    }
#pragma unroll
    for (int c = 0; c < ld; ++c)
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) acc[c] += __shfl_xor_sync(0xffffffffu, acc[c], o);
    if (lane == 0) {
      const double s = scale[row];
      y[row] = uref[row] + s * (double)(acc[0] + b3[row]);
#pragma unroll
      for (int c = 0; c < K; ++c) D[row * K + c] = s * (double)acc[1 + c];
    }
  }
}

template <int K>
__device__ void lspg_solve_block(int nblocks, const double *__restrict__ partial, double *__restrict__ x, double tol,
                                 int first, Flags *f);

// ---------------------------------------------------- LSPG residual / normal eqs
// Block of RB sample dof rows; thread (row, c) for c < K forms JR[row][c] =
// cf (Jf D)[row][c] + D[row][c] (its CSR row against column c of D), thread
// (row, K) the residual R[row]; then this block's partial sums of the upper
// triangle of JR^T JR, of JR^T R and of R^T R, each in a fixed row order.
__host__ __device__ constexpr int rows_per_block(int K) { return (K + 1) * 32 <= 1024 ? 32 : 16; }

template <int K>
__global__ void __launch_bounds__(rows_per_block(K) * (K + 1))
k_lspg_rows(int ndpc, long ns, const int *__restrict__ s2st, const double *__restrict__ y,
            const double *__restrict__ D, const double *__restrict__ V, const int *__restrict__ rowptr,
            const int *__restrict__ colidx, const double *__restrict__ J, double cf, double *__restrict__ yn,
            int first, double *__restrict__ partial, unsigned *__restrict__ ticket, double *__restrict__ x,
            double tol, Flags *f, double cn, double cnm1, double *__restrict__ ynm1, int bdf2) {
  if (!first && f->converged) return;
  constexpr int RB = rows_per_block(K);
  __shared__ double sJR[RB][K + 1];  // column K holds R
  const int t = threadIdx.x;
  const int rl = t / (K + 1), c = t % (K + 1);
  const long r = (long)blockIdx.x * RB + rl;
  double val = 0.;
  if (r < ns) {
    const long st = (long)s2st[r / ndpc] * ndpc + r % ndpc;  // stencil dof of this sample dof
    if (c == K) {
      const double ynp1 = y[st];
      if (first) {  // first iteration of a step: y_n-1 = y_n, y_n = y(x_n)
        ynm1[r] = yn[r];
        yn[r] = ynp1;
      }
      const double helper = bdf2 ? 1. * ynp1 + cn * yn[r] + cnm1 * ynm1[r] : 1. * ynp1 + cn * yn[r];
      val = cf * V[r] + 1. * helper;
    } else {
      double jd = 0.;
      const int q0 = rowptr[r], q1 = rowptr[r + 1];
      int q = q0;
      for (; q + 3 < q1; q += 4) {
        // the four column indices and products' operands loaded before the sums
        int ci[4];
        double jv[4], dv[4];
#pragma unroll
        for (int u = 0; u < 4; ++u) {
          ci[u] = __ldg(colidx + q + u);
          jv[u] = __ldg(J + q + u);
        }
#pragma unroll
        for (int u = 0; u < 4; ++u) dv[u] = __ldg(D + (long)ci[u] * K + c);
#pragma unroll
        for (int u = 0; u < 4; ++u) jd = fma(jv[u], dv[u], jd);
      }
      for (; q < q1; ++q) jd = fma(J[q], D[(long)colidx[q] * K + c], jd);
      val = fma(cf, jd, D[st * K + c]);
    }
  }
  sJR[rl][c] = val;
  __syncthreads();
  constexpr int ntri = K * (K + 1) / 2, ne = ntri + K + 1;
  for (int e = t; e < ne; e += blockDim.x) {
    int a, b;
    if (e < ntri) {
      a = 0;
      int rem = e;
      while (rem >= K - a) {
        rem -= K - a;
        ++a;
      }
      b = a + rem;
    } else if (e < ntri + K) {
      a = e - ntri;
      b = K;
    } else {
      a = K;
      b = K;
    }
    double s = 0.;
    for (int i = 0; i < RB; ++i) s = fma(sJR[i][a], sJR[i][b], s);
    partial[(long)blockIdx.x * ne + e] = s;
  }
  // the last block to finish reduces the partial sums and solves (ticket
  // counter; no block waits for another)
  __shared__ unsigned last;
  __threadfence();
  __syncthreads();
  if (t == 0) last = atomicAdd(ticket, 1u) == gridDim.x - 1 ? 1u : 0u;
  __syncthreads();
  if (!last) return;
  __threadfence();
  lspg_solve_block<K>((int)gridDim.x, partial, x, tol, first, f);
  if (t == 0) *ticket = 0u;
}

// Reduce the partial sums in block order, factor, solve, update.  GB300's
// FP64 units give one warp one instruction per ~64 cycles, so the k x k solve
// is arranged for a short dependency chain rather than few operations: a
// right-looking Cholesky in one warp (per column one reciprocal square root,
// the column scaled by it, the trailing triangle updated with the pairs spread
// over the lanes), then forward and backward substitution with one lane per
// unknown, multiplying by the stored reciprocal diagonal.  No division.
template <int K>
__device__ void lspg_solve_block(int nblocks, const double *__restrict__ partial, double *__restrict__ x, double tol,
                                 int first, Flags *f) {
  static_assert(K <= 32, "one lane per unknown");
  __shared__ double H[K][K];
  __shared__ double g[K];
  __shared__ double rdiag[K];
  __shared__ double rr;
  __shared__ unsigned char pi[K * (K + 1) / 2], pl[K * (K + 1) / 2];
  constexpr int ntri = K * (K + 1) / 2, ne = ntri + K + 1;
  const int lane = threadIdx.x & 31;
  // lower-triangle pairs (i, l), i >= l, ordered by l descending: the pairs
  // with l > j are the first (K-1-j)(K-j)/2 entries
  for (int q = threadIdx.x; q < ntri; q += blockDim.x) {
    int l = K - 1, rem = q;
    while (rem >= K - l) {
      rem -= K - l;
      --l;
    }
    pi[q] = (unsigned char)(l + rem);
    pl[q] = (unsigned char)l;
  }
  for (int e = threadIdx.x; e < ne; e += blockDim.x) {
    // one thread per entry, blocks in order, loads issued four at a time
    double s = 0.;
    int b = 0;
    for (; b + 4 <= nblocks; b += 4) {
      const double v0 = partial[(long)b * ne + e], v1 = partial[(long)(b + 1) * ne + e],
                   v2 = partial[(long)(b + 2) * ne + e], v3 = partial[(long)(b + 3) * ne + e];
      s += v0;
      s += v1;
      s += v2;
      s += v3;
    }
    for (; b < nblocks; ++b) s += partial[(long)b * ne + e];
    if (e < ntri) {
      int a = 0, rem = e;
      while (rem >= K - a) {
        rem -= K - a;
        ++a;
      }
      const int b2 = a + rem;
      H[a][b2] = s;
      H[b2][a] = s;
    } else if (e < ntri + K) {
      g[e - ntri] = s;
    } else {
      rr = s;
    }
  }
  __syncthreads();
  if (threadIdx.x < 32) {
    bool ok = true;
    for (int j = 0; j < K; ++j) {
      const double d = H[j][j];
      if (!(d > 0.)) {
        ok = false;
        break;
      }
      const double rs = rsqrt(d);
      if (lane == 0) rdiag[j] = rs;
      for (int i = j + 1 + lane; i < K; i += 32) H[i][j] *= rs;
      __syncwarp();
      const int np = (K - 1 - j) * (K - j) / 2;
      for (int q = lane; q < np; q += 32) {
        const int i = pi[q], l = pl[q];
        H[i][l] = fma(-H[i][j], H[l][j], H[i][l]);
      }
      __syncwarp();
    }
    // L z = g (lane i holds unknown i), then L^T dx = z
    double sv = lane < K ? g[lane] : 0.;
    double corr = 0.;
    if (ok) {
      for (int i = 0; i < K; ++i) {
        const double zi = __shfl_sync(0xffffffffu, sv, i) * rdiag[i];
        if (lane == i) sv = zi;
        if (lane > i && lane < K) sv = fma(-H[lane][i], zi, sv);
      }
      for (int i = K - 1; i >= 0; --i) {
        const double di = __shfl_sync(0xffffffffu, sv, i) * rdiag[i];
        if (lane == i) sv = di;
        if (lane < i) sv = fma(-H[i][lane], di, sv);
      }
      if (lane < K) x[lane] -= sv;
      double c2 = lane < K ? sv * sv : 0.;
#pragma unroll
      for (int o = 16; o > 0; o >>= 1) c2 += __shfl_xor_sync(0xffffffffu, c2, o);
      corr = c2;
    }
    if (lane == 0) {
      // the first iteration of a step starts the step's count and flag
      f->iters = first ? 1 : f->iters + 1;
      f->lastCorr = sqrt(corr);
      f->lastRes = sqrt(rr);
      if (!(f->lastRes <= f->maxRes)) f->maxRes = f->lastRes;
      f->converged = (!ok || sqrt(corr) < tol) ? 1 : 0;
    }
  }
}

}  // namespace rom
}  // namespace pda

// ------------------------------------------------------------------ object
struct pda_lspg {
  pda_problem *P = nullptr;
  int kind = 0;  // 0 affine, 1 MLP decoder
  int k = 0, ndpc = 0, h1 = 0, h2 = 0;
  long nst = 0, ns = 0, nSampleCells = 0;
  pda::DevBuf<int> s2st;
  pda::DevBuf<double> uref, phi, scale;
  pda::DevBuf<float> W1, b1, W2, b2, W3, b3, Z;
  bool tensorCore = false;
  pda::DevBuf<__nv_bfloat16> W3b, Zb;
  pda::DevBuf<double> y, D, V, J, yn, ynm1, partial, xn;
  pda::DevBuf<pda::rom::Flags> flags;
  pda::DevBuf<unsigned> ticket;
  int nblocks = 0;
  int64_t nnz = 0;
  // fused iteration (lspg_fused.cuh) or the assembled Jacobian path
  // (sample-mesh V + CSR J, then k_lspg_rows)
  bool fused = true;
  bool jac32 = false;  // fused form: single-precision Jacobian terms
  int fusedBlocks = 0;
  // one captured step per backward-difference formula: [0] BDF1 (also the
  // first step of a BDF2 trajectory), [1] BDF2
  struct StepGraph {
    cudaGraphExec_t exec = nullptr;
    double dt = 0;
    double *x = nullptr;
    int iters = 0;
    double tol = 0;
  } graph[2];
  void drop_graphs() {
    for (auto &g : graph)
      if (g.exec) {
        cudaGraphExecDestroy(g.exec);
        g.exec = nullptr;
      }
  }
  ~pda_lspg() { drop_graphs(); }
};

namespace pda {
namespace rom {
namespace {

int decode_grid(long nst) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  if (sms <= 0) sms = 1;
  return (int)std::min<long>(div_up(nst, 8), 2L * sms);
}

template <int K>
void decode_k(pda_lspg &L, const double *x, double *y, int first, cudaStream_t s) {
  Flags *f = L.flags.p;
  if (L.kind == 0) {
    k_decode_affine<K><<<div_up(L.nst, 256), 256, 0, s>>>(L.nst, L.uref.p, L.phi.p, x, y, first, f);
  } else if (L.tensorCore) {
    k_decode_hidden<K, 256><<<div_up(L.h2, kHiddenWarps), kHiddenWarps * 32, 0, s>>>(
        L.h2, L.W1.p, L.b1.p, L.W2.p, L.b2.p, x, L.Z.p, L.Zb.p, first, f);
    tc::ThinDecode dec;
    dec.b3 = L.b3.p;
    dec.uref = L.uref.p;
    dec.scale = L.scale.p;
    dec.y = y;
    dec.D = L.D.p;
    dec.K = K;
    PDA_CUDA(tc_gemm_thin_decode(L.W3b.p, L.Zb.p, L.nst, L.h2, dec, s));
  } else {
    k_decode_hidden<K, 256><<<div_up(L.h2, kHiddenWarps), kHiddenWarps * 32, 0, s>>>(
        L.h2, L.W1.p, L.b1.p, L.W2.p, L.b2.p, x, L.Z.p, nullptr, first, f);
    const int smem = L.h2 * (1 + K) * (int)sizeof(float);
    k_decode_out<K><<<decode_grid(L.nst), 256, smem, s>>>(L.h2, L.nst, L.W3.p, L.b3.p, L.uref.p, L.scale.p, L.Z.p,
                                                            y, L.D.p, first, f);
  }
}

// the backward-difference scheme of one step: BDF1 (c_n = -1, c_f = -1) or
// BDF2 (c_n = -4/3, c_n-1 = 1/3, c_f = -2/3), ode_constants.hpp:57-73
struct Bdf {
  double cf, cn, cnm1;
  int two;
};
inline Bdf bdf_coeffs(int order, double dt) {
  constexpr double one = 1., two = 2., three = 3., four = 4.;
  if (order == 2) return Bdf{-1. * (two / three) * dt, -1. * (four / three), one / three, 1};
  return Bdf{-1. * dt, -1., 0., 0};
}

template <int K>
void gn_iteration_k(pda_lspg &L, double *x, const Bdf &b, double tol, int first, cudaStream_t s) {
  Flags *f = L.flags.p;
  decode_k<K>(L, x, L.y.p, first, s);
  if (L.fused) {
    pda_problem &P = *L.P;
    LspgArgs a{L.y.p, L.D.p, K, b.cf, L.yn.p, first, L.V.p, L.partial.p, L.ticket.p, x, tol, f, L.jac32 ? 1 : 0};
    a.cn = b.cn;
    a.cnm1 = b.cnm1;
    a.ynm1 = L.ynm1.p;
    a.bdf2 = b.two;
    MeshArgs ma = P.margs;
    ma.time = 0.0;
    P.L->lspg_fused(P.scheme, P.innerT.t, P.nearT.t, ma, P.phys, a, s);
    PDA_CUDA(cudaGetLastError());
    return;
  }
  // sample-mesh velocity and Jacobian at y (the library's own kernels); they
  // run unconditionally, cheap next to the rest once converged
  const pda_status st = pda_velocity_and_jacobian(L.P, L.y.p, 0.0, L.V.p, L.J.p);
  if (st != PDA_OK) throw Error(st, pda_last_error());
  k_lspg_rows<K><<<L.nblocks, rows_per_block(K) * (K + 1), 0, s>>>(L.ndpc, L.ns, L.s2st.p, L.y.p, L.D.p, L.V.p,
                                                      L.P->d_rowptr.p, L.P->d_colidx.p, L.J.p, b.cf, L.yn.p, first,
                                                      L.partial.p, L.ticket.p, x, tol, f, b.cn, b.cnm1, L.ynm1.p,
                                                      b.two);
}

#define PDA_ROM_K_SWITCH(k, CALL) \
  switch (k) {                    \
    case 2: CALL(2); break;       \
    case 4: CALL(4); break;       \
    case 6: CALL(6); break;       \
    case 8: CALL(8); break;       \
    case 10: CALL(10); break;     \
    case 12: CALL(12); break;     \
    case 16: CALL(16); break;     \
    case 20: CALL(20); break;     \
    case 24: CALL(24); break;     \
    case 32: CALL(32); break;     \
    default: throw Error(PDA_ERR_UNSUPPORTED, "latent dimension not compiled"); \
  }

bool k_supported(int k) {
  return k == 2 || k == 4 || k == 6 || k == 8 || k == 10 || k == 12 || k == 16 || k == 20 || k == 24 || k == 32;
}

void gn_iteration(pda_lspg &L, double *x, const Bdf &b, double tol, int first, cudaStream_t s) {
#define PDA_ROM_GN(K) gn_iteration_k<K>(L, x, b, tol, first, s)
  PDA_ROM_K_SWITCH(L.k, PDA_ROM_GN)
#undef PDA_ROM_GN
}

void decode(pda_lspg &L, const double *x, double *y, cudaStream_t s) {
#define PDA_ROM_DEC(K) decode_k<K>(L, x, y, 1, s)
  PDA_ROM_K_SWITCH(L.k, PDA_ROM_DEC)
#undef PDA_ROM_DEC
}

void bdf_step(pda_lspg &L, double *x, const Bdf &b, double tol, int iters, cudaStream_t s) {
  // the first iteration ignores the previous step's convergence flag and resets it
  for (int it = 0; it < iters; ++it) gn_iteration(L, x, b, tol, it == 0 ? 1 : 0, s);
  PDA_CUDA(cudaGetLastError());
}

void common_setup(pda_lspg &L, pda_problem *P, const int64_t *s2st, int k) {
  PDA_REQUIRE(P && s2st, PDA_ERR_INVALID_ARGUMENT, "null argument");
  PDA_REQUIRE(k_supported(k), PDA_ERR_UNSUPPORTED,
              "latent dimension must be one of 2, 4, 6, 8, 10, 12, 16, 20, 24, 32");
  PDA_REQUIRE(!P->timeDependent, PDA_ERR_UNSUPPORTED,
              "LSPG steps evaluate the residual at a fixed time: problems with time-dependent ghost states "
              "(double Mach reflection) are not supported");
  L.P = P;
  L.k = k;
  L.ndpc = P->ndpc;
  L.nst = P->dofsStencil;
  L.ns = P->dofsSample;
  L.nSampleCells = L.ns / L.ndpc;
  std::vector<int> m((size_t)L.nSampleCells);
  for (long i = 0; i < L.nSampleCells; ++i) {
    PDA_REQUIRE(s2st[i] >= 0 && s2st[i] < L.nst / L.ndpc, PDA_ERR_INVALID_ARGUMENT,
                "sample-to-stencil index out of range");
    m[(size_t)i] = (int)s2st[i];
  }
  L.s2st.upload(m);
  int64_t rows = 0, cols = 0, nnz = 0;
  pda_status st = pda_jacobian_shape(P, &rows, &cols, &nnz);
  if (st != PDA_OK) throw Error(st, pda_last_error());
  L.nnz = nnz;
  L.y.alloc((size_t)L.nst);
  L.D.alloc((size_t)L.nst * k);
  L.V.alloc((size_t)L.ns);
  L.J.alloc((size_t)std::max<int64_t>(nnz, 1));
  L.yn.alloc((size_t)L.ns);
  L.ynm1.alloc((size_t)L.ns);
  L.nblocks = div_up(L.ns, rows_per_block(k));
  pda::ensure_row_tables(*P);
  P->L->lspg_fused_prepare();
  PDA_CUDA(cudaGetLastError());
  L.fusedBlocks = P->L->lspg_fused_blocks(P->scheme, P->innerT.t.nrows, P->nearT.t.nrows, k);
  L.partial.alloc((size_t)std::max(L.nblocks, L.fusedBlocks + lspg_groups(L.fusedBlocks)) *
                  (k * (k + 1) / 2 + k + 1));
  L.flags.alloc(1);
  L.ticket.alloc((size_t)(1 + lspg_groups(L.fusedBlocks)));
  PDA_CUDA(cudaMemset(L.ticket.p, 0, L.ticket.n * sizeof(unsigned)));
  L.xn.alloc((size_t)k);
  PDA_CUDA(cudaMemset(L.flags.p, 0, sizeof(Flags)));
  PDA_CUDA(cudaMemset(L.y.p, 0, (size_t)L.nst * sizeof(double)));
  // build the sample problem's tables and CSR pattern now (they allocate)
  st = pda_velocity_and_jacobian(P, L.y.p, 0.0, L.V.p, L.J.p);
  if (st != PDA_OK) throw Error(st, pda_last_error());
  PDA_CUDA(cudaDeviceSynchronize());
}

template <class T> void upload_dev(DevBuf<T> &b, const T *d_src, size_t n) {
  b.alloc(n);
  PDA_CUDA(cudaMemcpy(b.p, d_src, n * sizeof(T), cudaMemcpyDeviceToDevice));
}

}  // namespace
}  // namespace rom
}  // namespace pda

using pda::Error;

extern "C" {

pda_status pda_lspg_create_affine(pda_problem *sample_problem, const int64_t *sample_to_stencil, int k,
                                  const double *d_uref, const double *d_phi, pda_lspg **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(out && d_uref && d_phi, PDA_ERR_INVALID_ARGUMENT, "null argument");
  std::unique_ptr<pda_lspg> L(new pda_lspg);
  L->kind = 0;
  pda::rom::common_setup(*L, sample_problem, sample_to_stencil, k);
  pda::rom::upload_dev(L->uref, d_uref, (size_t)L->nst);
  pda::rom::upload_dev(L->phi, d_phi, (size_t)L->nst * k);
  // D is the constant basis
  PDA_CUDA(cudaMemcpy(L->D.p, d_phi, (size_t)L->nst * k * sizeof(double), cudaMemcpyDeviceToDevice));
  *out = L.release();
  PDA_API_END
}

pda_status pda_lspg_create_mlp(pda_problem *sample_problem, const int64_t *sample_to_stencil, int k, int h1,
                               int h2, const double *d_uref, const double *d_scale, const float *d_W1,
                               const float *d_b1, const float *d_W2, const float *d_b2, const float *d_W3,
                               const float *d_b3, int mode, pda_lspg **out) {
  PDA_API_BEGIN
  PDA_REQUIRE(out && d_uref && d_scale && d_W1 && d_b1 && d_W2 && d_b2 && d_W3 && d_b3, PDA_ERR_INVALID_ARGUMENT,
              "null argument");
  PDA_REQUIRE(h1 == 256, PDA_ERR_UNSUPPORTED, "decoder first hidden width must be 256");
  PDA_REQUIRE(h2 >= 1 && h2 * (1 + k) * (int)sizeof(float) <= 200 * 1024, PDA_ERR_UNSUPPORTED,
              "decoder second hidden width too large");
  std::unique_ptr<pda_lspg> L(new pda_lspg);
  L->kind = 1;
  L->h1 = h1;
  L->h2 = h2;
  pda::rom::common_setup(*L, sample_problem, sample_to_stencil, k);
  pda::rom::upload_dev(L->uref, d_uref, (size_t)L->nst);
  pda::rom::upload_dev(L->scale, d_scale, (size_t)L->nst);
  pda::rom::upload_dev(L->W1, d_W1, (size_t)h1 * k);
  pda::rom::upload_dev(L->b1, d_b1, (size_t)h1);
  pda::rom::upload_dev(L->W2, d_W2, (size_t)h2 * h1);
  PDA_CUDA(cudaGetLastError());
  PDA_CUDA(cudaDeviceSynchronize());
  pda::rom::upload_dev(L->b2, d_b2, (size_t)h2);
  pda::rom::upload_dev(L->W3, d_W3, (size_t)L->nst * h2);
  pda::rom::upload_dev(L->b3, d_b3, (size_t)L->nst);
  L->Z.alloc((size_t)h2 * (1 + k));
  if (mode == 1) {
    // bf16 output layer on the tensor cores: the weights must be bf16 values
    PDA_REQUIRE(h2 % 64 == 0 && k + 1 <= 16, PDA_ERR_UNSUPPORTED,
                "tensor-core decoder: hidden width a multiple of 64 and latent at most 15");
    L->tensorCore = true;
    // the weights in bf16, then blocked by 128-row tiles and 64-column slices
    // (rows past nst zero) so that each slice the GEMM reads is one block
    pda::DevBuf<__nv_bfloat16> w3rows;
    w3rows.alloc((size_t)L->nst * h2);
    L->W3b.alloc((size_t)pda::div_up(L->nst, 128) * 128 * h2);
    L->Zb.alloc((size_t)16 * h2);
    PDA_CUDA(cudaMemset(L->Zb.p, 0, (size_t)16 * h2 * sizeof(__nv_bfloat16)));
    pda::DevBuf<int> bad;
    bad.alloc(1);
    PDA_CUDA(cudaMemset(bad.p, 0, sizeof(int)));
    pda::rom::k_to_bf16_exact<<<pda::div_up(L->nst * (long)h2, 256), 256>>>(L->W3.p, w3rows.p, L->nst * (long)h2,
                                                                             bad.p);
    PDA_CUDA(cudaGetLastError());
    int hb = 0;
    PDA_CUDA(cudaMemcpy(&hb, bad.p, sizeof(int), cudaMemcpyDeviceToHost));
    PDA_REQUIRE(hb == 0, PDA_ERR_INVALID_ARGUMENT,
                "tensor-core decoder: output-layer weights are not bf16 values (use mode 0)");
    PDA_CUDA(pda::tc_block_operand(w3rows.p, L->nst, h2, 128, L->W3b.p, nullptr));
    // before any capture: the GEMM's shared-memory attribute
    PDA_CUDA(pda::tc_gemm_thin_prepare());
    PDA_CUDA(cudaDeviceSynchronize());
  } else {
    PDA_REQUIRE(mode == 0, PDA_ERR_INVALID_ARGUMENT, "mode must be 0 (fp32) or 1 (bf16 tensor cores)");
  }
  const int smem = h2 * (1 + k) * (int)sizeof(float);
  if (smem > 48 * 1024) {
#define PDA_ROM_ATTR(K) \
  PDA_CUDA(cudaFuncSetAttribute(pda::rom::k_decode_out<K>, cudaFuncAttributeMaxDynamicSharedMemorySize, smem))
    PDA_ROM_K_SWITCH(k, PDA_ROM_ATTR)
#undef PDA_ROM_ATTR
  }
  *out = L.release();
  PDA_API_END
}

void pda_lspg_free(pda_lspg *L) { delete L; }

pda_status pda_lspg_decode(pda_lspg *L, const double *d_x, double *d_y) {
  PDA_API_BEGIN
  PDA_REQUIRE(L && d_x && d_y, PDA_ERR_INVALID_ARGUMENT, "null argument");
  cudaStream_t s = L->P->stream;
  pda::rom::decode(*L, d_x, d_y, s);
  PDA_CUDA(cudaGetLastError());
  PDA_CUDA(cudaStreamSynchronize(s));
  PDA_API_END
}

pda_status pda_lspg_set_fused(pda_lspg *rom, int fused) {
  PDA_API_BEGIN
  PDA_REQUIRE(rom, PDA_ERR_INVALID_ARGUMENT, "null argument");
  if (rom->fused != (fused != 0)) rom->drop_graphs();
  rom->fused = fused != 0;
  PDA_API_END
}

pda_status pda_lspg_set_jacobian_precision(pda_lspg *rom, int bits) {
  PDA_API_BEGIN
  PDA_REQUIRE(rom && (bits == 32 || bits == 64), PDA_ERR_INVALID_ARGUMENT, "bits must be 32 or 64");
  if (rom->jac32 != (bits == 32)) rom->drop_graphs();
  rom->jac32 = bits == 32;
  PDA_API_END
}

pda_status pda_lspg_advance(pda_lspg *L, double *d_x, double dt, int64_t n_steps, int gn_iters, double tol,
                            int order, int64_t first_step, int use_graph, double *info) {
  PDA_API_BEGIN
  PDA_REQUIRE(L && d_x && n_steps >= 0 && gn_iters >= 1, PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  PDA_REQUIRE(order == 1 || order == 2, PDA_ERR_INVALID_ARGUMENT, "order must be 1 (BDF1) or 2 (BDF2)");
  PDA_REQUIRE(first_step >= 1, PDA_ERR_INVALID_ARGUMENT, "steps are numbered from 1");
  cudaStream_t s = L->P->stream;
  // info[3] covers this call's steps
  PDA_CUDA(cudaMemsetAsync(&L->flags.p->maxRes, 0, sizeof(double), s));
  for (int64_t n = 0; n < n_steps; ++n) {
    // Pressio's BDF2 LSPG takes its first step with BDF1 (lspg_unsteady_rj_policy_hypred.hpp:124-134)
    const int slot = (order == 2 && first_step + n > 1) ? 1 : 0;
    const pda::rom::Bdf b = pda::rom::bdf_coeffs(slot == 1 ? 2 : 1, dt);
    if (!use_graph || s == nullptr) {
      pda::rom::bdf_step(*L, d_x, b, tol, gn_iters, s);
      continue;
    }
    auto &G = L->graph[slot];
    if (G.exec && (G.dt != dt || G.x != d_x || G.iters != gn_iters || G.tol != tol)) {
      cudaGraphExecDestroy(G.exec);
      G.exec = nullptr;
    }
    if (!G.exec) {
      PDA_CUDA(cudaStreamSynchronize(s));
      cudaGraph_t g;
      PDA_CUDA(cudaStreamBeginCapture(s, cudaStreamCaptureModeThreadLocal));
      try {
        pda::rom::bdf_step(*L, d_x, b, tol, gn_iters, s);
      } catch (...) {
        cudaStreamEndCapture(s, &g);
        throw;
      }
      PDA_CUDA(cudaStreamEndCapture(s, &g));
      PDA_CUDA(cudaGraphInstantiate(&G.exec, g, 0));
      cudaGraphDestroy(g);
      G.dt = dt;
      G.x = d_x;
      G.iters = gn_iters;
      G.tol = tol;
    }
    PDA_CUDA(cudaGraphLaunch(G.exec, s));
  }
  if (info) {
    pda::rom::Flags hf;
    PDA_CUDA(cudaMemcpyAsync(&hf, L->flags.p, sizeof(hf), cudaMemcpyDeviceToHost, s));
    PDA_CUDA(cudaStreamSynchronize(s));
    info[0] = hf.lastCorr;
    info[1] = (double)hf.iters;
    info[2] = hf.lastRes;
    info[3] = hf.maxRes;
  }
  PDA_API_END
}

pda_status pda_lspg_advance_bdf1(pda_lspg *L, double *d_x, double dt, int64_t n_steps, int gn_iters, double tol,
                                 int use_graph, double *info) {
  return pda_lspg_advance(L, d_x, dt, n_steps, gn_iters, tol, 1, 1, use_graph, info);
}

}  // extern "C"
