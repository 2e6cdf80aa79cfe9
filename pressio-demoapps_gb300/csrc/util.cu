// Element-wise stepper updates, the CSR sparse x dense product, the FP64
// throughput probe and the self-checks of the integer-pipe division, square
// root and exact products.
#include "fp64_intpipe.cuh"
#include "launch.hpp"

namespace pda {
namespace {

// Stage updates with the association of Pressio's ops::update on Eigen
// vectors (tests_cpp/pressio/include/pressio/ops/eigen/ops_rank1_update.hpp:
// 26-46, 67-94, 179-215): v = a*v + b*x + c*y evaluated left to right, and
// v = b*x + c*y when a == 0.
__global__ void k_x_plus_ay(double *__restrict__ out, const double *__restrict__ x,
                            const double *__restrict__ y, double a, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) out[i] = x[i] + a * y[i];
}

__global__ void k_av_bx_cy(double *__restrict__ v, double a, const double *__restrict__ x, double b,
                           const double *__restrict__ y, double c, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = a * v[i] + b * x[i] + c * y[i];
}

__global__ void k_rk4_final(double *__restrict__ v, const double *__restrict__ r1,
                            const double *__restrict__ r2, const double *__restrict__ r3,
                            const double *__restrict__ r4, double dt6, double dt3, long n) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) v[i] = v[i] + dt6 * r1[i] + dt3 * r2[i] + dt3 * r3[i] + dt6 * r4[i];
}

// R(:,c) = J * B(:,c); per row the products are summed in CSR order from
// zero, as Eigen's row-major sparse * dense product does.
__global__ void k_csr_spmm(long rows, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                           const double *__restrict__ vals, const double *__restrict__ B, long ldb,
                           int ncols, double *__restrict__ R, long ldr) {
  const long t = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (t >= rows * ncols) return;
  const long r = t % rows;
  const long c = t / rows;
  double acc = 0.;
  for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) acc += vals[q] * B[c * ldb + colidx[q]];
  R[c * ldr + r] = acc;
}

// Independent DFMA chains per thread; 8 chains hide the pipeline latency.
__global__ void k_fp64_fma(double *out, int iters, double a, double b) {
  double x[8];
#pragma unroll
  for (int k = 0; k < 8; ++k) x[k] = threadIdx.x * 1e-7 + k;
  for (int i = 0; i < iters; ++i) {
#pragma unroll
    for (int k = 0; k < 8; ++k) x[k] = fma(x[k], a, b);
  }
  double s = 0;
#pragma unroll
  for (int k = 0; k < 8; ++k) s += x[k];
  if (s == 123.456) out[threadIdx.x] = s;  // keeps the chains alive
}

__device__ __forceinline__ uint64_t splitmix64(uint64_t &s) {
  uint64_t z = (s += 0x9E3779B97F4A7C15ull);
  z = (z ^ (z >> 30)) * 0xBF58476D1CE4E5B9ull;
  z = (z ^ (z >> 27)) * 0x94D049BB133111EBull;
  return z ^ (z >> 31);
}

// Operand sets for the comparison of ip::div / ip::sqrt with the FP64 pipe's
// IEEE operations.  mode 0: random mantissas, exponents within 2^-40..2^40
// (quotients and roots of the normal range); 1: divisors with mantissas
// within 1024 units of 1 and of 2 - 2^-52 (the ends of the reciprocal's
// range); 2: near-exact quotients and roots (rounding midpoints and exact
// results: a = b q or x = q^2 with short q, moved by up to two units);
// 3: arbitrary bit patterns (zeros, subnormals, infinities, NaNs included).
__global__ void k_check_divsqrt(int mode, uint64_t seed, long per_thread, unsigned long long *bad) {
  uint64_t st = seed ^ ((uint64_t)(blockIdx.x * blockDim.x + threadIdx.x) * 0x632BE59BD9B4E019ull);
  unsigned long long nd = 0, ns = 0;
  constexpr uint64_t M = 0x000FFFFFFFFFFFFFull;
  for (long k = 0; k < per_thread; ++k) {
    const uint64_t r1 = splitmix64(st), r2 = splitmix64(st), r3 = splitmix64(st);
    uint64_t ua, ub, ux;
    if (mode == 0) {
      ua = (r1 & M) | ((uint64_t)(1023 + (int)(r3 % 81) - 40) << 52) | (r3 & (1ull << 63));
      ub = (r2 & M) | ((uint64_t)(1023 + (int)((r3 >> 8) % 81) - 40) << 52) | ((r3 << 1) & (1ull << 63));
      ux = (r2 & M) | ((uint64_t)(1023 - 60 + (int)((r1 >> 52) % 121)) << 52);
    } else if (mode == 1) {
      const uint64_t m = (r2 & 1) ? (M - (r2 >> 1) % 1024) : ((r2 >> 1) % 1024);
      ua = (r1 & M) | (1023ull << 52);
      ub = m | ((uint64_t)(1000 + (r3 % 40)) << 52);
      ux = m | ((uint64_t)(1000 + (r3 % 41)) << 52);
    } else if (mode == 2) {
      const double b = __longlong_as_double((long long)((r2 & M & ~0xFFFFFFull) | (1023ull << 52)));
      const double q = __longlong_as_double((long long)((r1 & M & ~0xFFFFFFFull) | (1023ull << 52)));
      ua = (uint64_t)__double_as_longlong(b * q) + (r3 & 1 ? ((r3 >> 1) % 5) - 2 : 0);
      ub = (uint64_t)__double_as_longlong(b);
      ux = (uint64_t)__double_as_longlong(q * q) + ((r3 >> 8) % 5) - 2;
    } else {
      ua = r1;
      ub = r2;
      ux = r3;
    }
    const double a = __longlong_as_double((long long)ua), b = __longlong_as_double((long long)ub);
    const double x = __longlong_as_double((long long)ux);
    const double hd = a / b, gd = ip::div(a, b);
    const double hs = sqrt(x), gs = ip::sqrt(x);
    nd += !(__double_as_longlong(hd) == __double_as_longlong(gd) || (hd != hd && gd != gd));
    ns += !(__double_as_longlong(hs) == __double_as_longlong(gs) || (hs != hs && gs != gs));
  }
  atomicAdd(bad, nd);
  atomicAdd(bad + 1, ns);
}

// Operand sets for the comparison of the integer-pipe products by constants
// (ip::mul_small<K>, ip::mul_pow2_neg<S>, ip::mul_const) and of
// ip::add_1em30 with the FP64
// pipe's operations.  mode 0: random mantissas, exponents within 2^-60..2^60;
// 1: exponents at the edges of the fast paths (subnormal results of the
// halvings, near-overflow products, the 2^-44 bound of the density guard)
// and short mantissas (exact products and rounding ties); 2: mantissas
// within 64 units of 1 and of 2 - 2^-52; 3: arbitrary bit patterns (zeros,
// subnormals, infinities, NaNs included).
__device__ __forceinline__ bool same_bits(double a, double b) {
  return __double_as_longlong(a) == __double_as_longlong(b) || (a != a && b != b);
}

__global__ void k_check_products(int mode, uint64_t seed, long per_thread, unsigned long long *bad) {
  uint64_t st = seed ^ ((uint64_t)(blockIdx.x * blockDim.x + threadIdx.x) * 0x9E6C63D0676A9A99ull);
  unsigned long long nk = 0, np = 0, ne = 0, nc = 0;
  constexpr uint64_t M = 0x000FFFFFFFFFFFFFull;
  for (long k = 0; k < per_thread; ++k) {
    const uint64_t r1 = splitmix64(st), r2 = splitmix64(st);
    uint64_t ux;
    if (mode == 0) {
      ux = (r1 & M) | ((uint64_t)(1023 - 60 + (int)(r2 % 121)) << 52) | (r2 & (1ull << 63));
    } else if (mode == 1) {
      static const int edges[] = {0, 1, 2, 3, 4, 0x7F5, 0x7F6, 0x7F7, 0x7F8, 0x7F9, 0x7FA, 0x7FB, 0x7FE, 0x7FF,
                                  975, 976, 977, 978, 979, 980, 981, 1023};
      const int e = edges[(r2 >> 8) % (sizeof(edges) / sizeof(edges[0]))];
      const uint64_t m = (r2 & 1) ? (r1 & M & ~((1ull << 40) - 1)) : (r1 & M);
      ux = m | ((uint64_t)e << 52) | (r2 & (1ull << 63));
    } else if (mode == 2) {
      const uint64_t m = (r2 & 1) ? (M - (r2 >> 1) % 64) : ((r2 >> 1) % 64);
      ux = m | ((uint64_t)(1000 + (r1 % 48)) << 52) | (r1 & (1ull << 63));
    } else {
      ux = r1;
    }
    const double x = __longlong_as_double((long long)ux);
    nk += !same_bits(x * 3., ip::mul_small<3>(x));
    nk += !same_bits(x * 5., ip::mul_small<5>(x));
    nk += !same_bits(x * 7., ip::mul_small<7>(x));
    nk += !same_bits(x * 11., ip::mul_small<11>(x));
    nk += !same_bits(x * 13., ip::mul_small<13>(x));
    np += !same_bits(x * 0.5, ip::mul_pow2_neg<1>(x));
    np += !same_bits(x * 0.25, ip::mul_pow2_neg<2>(x));
    ne += !same_bits(x + 1.e-30, ip::add_1em30(x));
    nc += !same_bits(x * (1. / 6.), ip::mul_const(x, 1. / 6.));
    nc += !same_bits(x * (13. / 12.), ip::mul_const(x, 13. / 12.));
    nc += !same_bits(x * (2. * 1e-6), ip::mul_const(x, 2. * 1e-6));
    nc += !same_bits(x * 0.1, ip::mul_const(x, 0.1));
    nc += !same_bits(x * 1.4, ip::mul_const(x, 1.4));
    nc += !same_bits(x * 1e300, ip::mul_const(x, 1e300));
    nc += !same_bits(x * 1e-300, ip::mul_const(x, 1e-300));
  }
  atomicAdd(bad, nk);
  atomicAdd(bad + 1, np);
  atomicAdd(bad + 2, ne);
  atomicAdd(bad + 3, nc);
}

}  // namespace

void check_divsqrt(int mode, uint64_t seed, long per_thread, long long counts[3], cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  unsigned long long *bad = nullptr;
  cudaMalloc((void **)&bad, 2 * sizeof(unsigned long long));
  cudaMemsetAsync(bad, 0, 2 * sizeof(unsigned long long), s);
  const int blocks = (sms > 0 ? sms : 1) * 8, threads = 256;
  k_check_divsqrt<<<blocks, threads, 0, s>>>(mode, seed, per_thread, bad);
  unsigned long long h[2] = {0, 0};
  cudaMemcpyAsync(h, bad, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  cudaFree(bad);
  counts[0] = (long long)blocks * threads * per_thread;
  counts[1] = (long long)h[0];
  counts[2] = (long long)h[1];
}

void check_products(int mode, uint64_t seed, long per_thread, long long counts[5], cudaStream_t s) {
  int dev = 0, sms = 0;
  cudaGetDevice(&dev);
  cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
  unsigned long long *bad = nullptr;
  cudaMalloc((void **)&bad, 4 * sizeof(unsigned long long));
  cudaMemsetAsync(bad, 0, 4 * sizeof(unsigned long long), s);
  const int blocks = (sms > 0 ? sms : 1) * 8, threads = 256;
  k_check_products<<<blocks, threads, 0, s>>>(mode, seed, per_thread, bad);
  unsigned long long h[4] = {0, 0, 0, 0};
  cudaMemcpyAsync(h, bad, sizeof(h), cudaMemcpyDeviceToHost, s);
  cudaStreamSynchronize(s);
  cudaFree(bad);
  counts[0] = (long long)blocks * threads * per_thread;
  counts[1] = (long long)h[0];
  counts[2] = (long long)h[1];
  counts[3] = (long long)h[2];
  counts[4] = (long long)h[3];
}

double measure_fp64_fma_rate(int blocks, int threads, int iters, cudaStream_t s) {
  double *out = nullptr;
  cudaMalloc((void **)&out, sizeof(double) * threads);
  cudaEvent_t e0, e1;
  cudaEventCreate(&e0);
  cudaEventCreate(&e1);
  k_fp64_fma<<<blocks, threads, 0, s>>>(out, iters / 10, 0.999999, 1e-7);  // warm-up
  cudaEventRecord(e0, s);
  k_fp64_fma<<<blocks, threads, 0, s>>>(out, iters, 0.999999, 1e-7);
  cudaEventRecord(e1, s);
  cudaEventSynchronize(e1);
  float ms = 0;
  cudaEventElapsedTime(&ms, e0, e1);
  cudaEventDestroy(e0);
  cudaEventDestroy(e1);
  cudaFree(out);
  const double flops = 2.0 * 8.0 * (double)iters * (double)blocks * (double)threads;
  return flops / (ms * 1e-3);
}

// kind 0: out = a + cb*b
// kind 1: out = ca*out + cb*a + cc*b
// kind 2: out = out + cd*a + cb*b + cb*c + cd*d   (RK4 final; cd = dt/6, cb = dt/3)
void launch_axpby_stage(int kind, double *out, const double *a, const double *b, const double *c,
                        double ca, double cb, double cc, double cd, const double *d,
                        const double * /*e*/, long n, cudaStream_t s) {
  const int g = div_up(n, 256);
  if (kind == 0) k_x_plus_ay<<<g, 256, 0, s>>>(out, a, b, cb, n);
  else if (kind == 1) k_av_bx_cy<<<g, 256, 0, s>>>(out, ca, a, cb, b, cc, n);
  else k_rk4_final<<<g, 256, 0, s>>>(out, a, b, c, d, cd, cb, n);
}

void launch_csr_spmm(long rows, const int *rowptr, const int *colidx, const double *vals, const double *B,
                     long ldb, int ncols, double *R, long ldr, cudaStream_t s) {
  const long n = rows * (long)ncols;
  if (n <= 0) return;
  k_csr_spmm<<<div_up(n, 128), 128, 0, s>>>(rows, rowptr, colidx, vals, B, ldb, ncols, R, ldr);
}

}  // namespace pda
