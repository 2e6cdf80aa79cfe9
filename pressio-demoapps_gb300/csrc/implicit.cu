// Implicit time integration on the device: BDF1 or Crank-Nicolson steps
// solved by Newton-Raphson, each correction by BiCGSTAB with a Jacobi
// (diagonal) preconditioner on the device CSR Jacobian -- the consumer of
// the reference's Jacobian in its implicit tests
// (tests_cpp/eigen_2d_euler_riemann_implicit/main.cc:31-44: Pressio's
// implicit stepper, create_newton_solver, iterative::Bicgstab).
//
// Step n -> n+1 with f the velocity (ode_constants.hpp):
//   BDF1  R(y) = y - y_n - dt f(y)                    J_R = I - dt Jf(y)
//   CN    R(y) = y - y_n - dt/2 (f(y) + f(y_n))       J_R = I - dt/2 Jf(y)
// Newton (nonlinear_least_squares.hpp:50-112): per iteration R and J_R at y,
// solve J_R d = R, stop before updating when |d|_2 < tol (Pressio's default
// criterion, the absolute l2 norm of the correction), else y <- y - d.
// BiCGSTAB follows the standard preconditioned algorithm (van der Vorst)
// that Eigen's BiCGSTAB implements, with the scalars kept on the device and
// reductions in a fixed order.
#include <cmath>
#include <cstdint>
#include <string>
#include <vector>

#include <cuda_runtime.h>

#include "problem_impl.hpp"

namespace pda {
namespace impl {

constexpr int RB = 256;      // threads per reduction block
constexpr int NRED = 1024;   // reduction blocks (grid-stride)

// ----------------------------------------------------------- vector kernels
__global__ void k_residual(int scheme, long n, const double *__restrict__ y, const double *__restrict__ yn,
                           const double *__restrict__ f, const double *__restrict__ fn, double dt,
                           double *__restrict__ R) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  if (scheme == 0) R[i] = y[i] - yn[i] - dt * f[i];
  else R[i] = y[i] - yn[i] - (dt / 2.) * (f[i] + fn[i]);
}

// J_R = I + c Jf in place of a copy of Jf's values; diag[i] = J_R(i, i)
__global__ void k_jr_values(long rows, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                            const double *__restrict__ J, double c, double *__restrict__ JR,
                            double *__restrict__ diag) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double d = 1.;
  for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) {
    double v = c * J[q];
    if (colidx[q] == r) {
      v += 1.;
      d = v;
    }
    JR[q] = v;
  }
  diag[r] = d;
}

__global__ void k_spmv(long rows, const int *__restrict__ rowptr, const int *__restrict__ colidx,
                       const double *__restrict__ A, const double *__restrict__ x, double *__restrict__ y) {
  const long r = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (r >= rows) return;
  double s = 0.;
  for (int q = rowptr[r]; q < rowptr[r + 1]; ++q) s += A[q] * x[colidx[q]];
  y[r] = s;
}

// block partial sums of a.b (fixed order inside each block)
__global__ void __launch_bounds__(RB) k_dot_partial(long n, const double *__restrict__ a,
                                                    const double *__restrict__ b, double *__restrict__ part) {
  __shared__ double red[RB];
  double s = 0.;
  for (long i = (long)blockIdx.x * RB + threadIdx.x; i < n; i += (long)gridDim.x * RB) s += a[i] * b[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = RB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) part[blockIdx.x] = red[0];
}

// out = sum of the partials (one block)
__global__ void __launch_bounds__(RB) k_dot_final(int nparts, const double *__restrict__ part, double *out) {
  __shared__ double red[RB];
  double s = 0.;
  for (int i = threadIdx.x; i < nparts; i += RB) s += part[i];
  red[threadIdx.x] = s;
  __syncthreads();
  for (int o = RB / 2; o > 0; o >>= 1) {
    if (threadIdx.x < o) red[threadIdx.x] += red[threadIdx.x + o];
    __syncthreads();
  }
  if (threadIdx.x == 0) *out = red[0];
}

// scalar slots of the solver state on the device
enum Sc { RHO, RHO_OLD, ALPHA, OMEGA, BETA, R0V, TT, TS, RR, BB, NSC };

__global__ void k_beta(double *sc) {
  // beta = (rho / rho_old) * (alpha / omega)
  sc[BETA] = (sc[RHO] / sc[RHO_OLD]) * (sc[ALPHA] / sc[OMEGA]);
}
__global__ void k_alpha(double *sc) { sc[ALPHA] = sc[RHO] / sc[R0V]; }
__global__ void k_omega(double *sc) { sc[OMEGA] = sc[TT] > 0. ? sc[TS] / sc[TT] : 0.; }
__global__ void k_shift_rho(double *sc) { sc[RHO_OLD] = sc[RHO]; }

// p = r + beta (p - omega v);  y = p / diag
__global__ void k_update_p(long n, const double *__restrict__ r, const double *__restrict__ v,
                           const double *__restrict__ diag, const double *__restrict__ sc, double *__restrict__ p,
                           double *__restrict__ y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double pi = r[i] + sc[BETA] * (p[i] - sc[OMEGA] * v[i]);
  p[i] = pi;
  y[i] = pi / diag[i];
}

// s = r - alpha v;  z = s / diag
__global__ void k_update_s(long n, const double *__restrict__ r, const double *__restrict__ v,
                           const double *__restrict__ diag, const double *__restrict__ sc, double *__restrict__ s,
                           double *__restrict__ z) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double si = r[i] - sc[ALPHA] * v[i];
  s[i] = si;
  z[i] = si / diag[i];
}

// x += alpha y + omega z;  r = s - omega t
__global__ void k_update_xr(long n, const double *__restrict__ y, const double *__restrict__ z,
                            const double *__restrict__ s, const double *__restrict__ t,
                            const double *__restrict__ sc, double *__restrict__ x, double *__restrict__ r) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i >= n) return;
  x[i] += sc[ALPHA] * y[i] + sc[OMEGA] * z[i];
  r[i] = s[i] - sc[OMEGA] * t[i];
}

__global__ void k_copy(long n, const double *__restrict__ a, double *__restrict__ b) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = a[i];
}
__global__ void k_fill(long n, double v, double *__restrict__ b) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) b[i] = v;
}
__global__ void k_axpy(long n, double a, const double *__restrict__ x, double *__restrict__ y) {
  const long i = (long)blockIdx.x * blockDim.x + threadIdx.x;
  if (i < n) y[i] += a * x[i];
}

struct Work {
  DevBuf<double> Un, Vn, V, J, JR, diag, R, d, r, r0, p, v, s, t, y, z, part, sc;
};

unsigned g1(long n) { return (unsigned)((n + 255) / 256); }

void dot(Work &w, long n, const double *a, const double *b, int slot, cudaStream_t st) {
  k_dot_partial<<<NRED, RB, 0, st>>>(n, a, b, w.part.p);
  k_dot_final<<<1, RB, 0, st>>>(NRED, w.part.p, w.sc.p + slot);
}

double read_scalar(Work &w, int slot, cudaStream_t st) {
  double h = 0.;
  PDA_CUDA(cudaMemcpyAsync(&h, w.sc.p + slot, sizeof(double), cudaMemcpyDeviceToHost, st));
  PDA_CUDA(cudaStreamSynchronize(st));
  return h;
}

// solve JR d = R (x0 = 0); returns iterations, relres in *relres
int bicgstab(Work &w, long n, const int *rowptr, const int *colidx, double tol, int maxIt, cudaStream_t st,
             double *relres) {
  double *x = w.d.p;
  k_fill<<<g1(n), 256, 0, st>>>(n, 0., x);
  k_copy<<<g1(n), 256, 0, st>>>(n, w.R.p, w.r.p);
  k_copy<<<g1(n), 256, 0, st>>>(n, w.R.p, w.r0.p);
  k_fill<<<g1(n), 256, 0, st>>>(n, 0., w.p.p);
  k_fill<<<g1(n), 256, 0, st>>>(n, 0., w.v.p);
  const double one = 1.;
  for (int s : {RHO, ALPHA, OMEGA})
    PDA_CUDA(cudaMemcpyAsync(w.sc.p + s, &one, sizeof(double), cudaMemcpyHostToDevice, st));
  dot(w, n, w.R.p, w.R.p, BB, st);
  const double bb = read_scalar(w, BB, st);
  if (!(bb > 0.)) {
    *relres = 0.;
    return 0;
  }
  int it = 0;
  double rr = bb;
  while (it < maxIt) {
    ++it;
    k_shift_rho<<<1, 1, 0, st>>>(w.sc.p);
    dot(w, n, w.r0.p, w.r.p, RHO, st);
    k_beta<<<1, 1, 0, st>>>(w.sc.p);
    k_update_p<<<g1(n), 256, 0, st>>>(n, w.r.p, w.v.p, w.diag.p, w.sc.p, w.p.p, w.y.p);
    k_spmv<<<g1(n), 256, 0, st>>>(n, rowptr, colidx, w.JR.p, w.y.p, w.v.p);
    dot(w, n, w.r0.p, w.v.p, R0V, st);
    k_alpha<<<1, 1, 0, st>>>(w.sc.p);
    k_update_s<<<g1(n), 256, 0, st>>>(n, w.r.p, w.v.p, w.diag.p, w.sc.p, w.s.p, w.z.p);
    k_spmv<<<g1(n), 256, 0, st>>>(n, rowptr, colidx, w.JR.p, w.z.p, w.t.p);
    dot(w, n, w.t.p, w.t.p, TT, st);
    dot(w, n, w.t.p, w.s.p, TS, st);
    k_omega<<<1, 1, 0, st>>>(w.sc.p);
    k_update_xr<<<g1(n), 256, 0, st>>>(n, w.y.p, w.z.p, w.s.p, w.t.p, w.sc.p, x, w.r.p);
    dot(w, n, w.r.p, w.r.p, RR, st);
    rr = read_scalar(w, RR, st);
    if (!(rr >= 0.) || rr <= tol * tol * bb) break;
  }
  PDA_CUDA(cudaGetLastError());
  *relres = std::sqrt(rr / bb);
  return it;
}

}  // namespace impl
}  // namespace pda

using pda::Error;

extern "C" {

pda_status pda_advance_implicit(pda_problem *p, double *d_U, double t0, double dt, int64_t n_steps, int scheme,
                                double newton_tol, int newton_max_iters, double linear_tol, int linear_max_iters,
                                double *info) {
  PDA_API_BEGIN
  PDA_REQUIRE(p && d_U && n_steps >= 0 && (scheme == 0 || scheme == 1) && newton_max_iters >= 1 &&
                  linear_max_iters >= 1,
              PDA_ERR_INVALID_ARGUMENT, "invalid argument");
  pda_problem &P = *p;
  PDA_REQUIRE(P.dofsSample == P.dofsStencil, PDA_ERR_UNSUPPORTED, "implicit time integration needs a full mesh");
  const long n = (long)P.dofsStencil;
  int64_t rows = 0, cols = 0, nnz = 0;
  pda_status st = pda_jacobian_shape(p, &rows, &cols, &nnz);
  if (st != PDA_OK) throw Error(st, pda_last_error());
  pda::impl::Work w;
  for (auto *b : {&w.Un, &w.Vn, &w.V, &w.diag, &w.R, &w.d, &w.r, &w.r0, &w.p, &w.v, &w.s, &w.t, &w.y, &w.z})
    b->alloc((size_t)n);
  w.J.alloc((size_t)nnz);
  w.JR.alloc((size_t)nnz);
  w.part.alloc(pda::impl::NRED);
  w.sc.alloc(pda::impl::NSC);
  cudaStream_t s = P.stream;
  pda::ensure_device_pattern(P);
  const int *rowptr = P.d_rowptr.p, *colidx = P.d_colidx.p;
  int totalNewton = 0, totalLinear = 0, maxNewton = 0;
  double worstRel = 0.;
  double t = t0;
  for (int64_t step = 0; step < n_steps; ++step) {
    pda::impl::k_copy<<<pda::impl::g1(n), 256, 0, s>>>(n, d_U, w.Un.p);
    if (scheme == 1) {
      st = pda_velocity(p, w.Un.p, t, w.Vn.p);
      if (st != PDA_OK) throw Error(st, pda_last_error());
    }
    const double c = scheme == 0 ? -dt : -dt / 2.;
    int it = 0;
    for (; it < newton_max_iters; ++it) {
      st = pda_velocity_and_jacobian(p, d_U, t + dt, w.V.p, w.J.p);
      if (st != PDA_OK) throw Error(st, pda_last_error());
      pda::impl::k_residual<<<pda::impl::g1(n), 256, 0, s>>>(scheme, n, d_U, w.Un.p, w.V.p, w.Vn.p, dt, w.R.p);
      pda::impl::k_jr_values<<<pda::impl::g1(n), 256, 0, s>>>(n, rowptr, colidx, w.J.p, c, w.JR.p, w.diag.p);
      double rel = 0.;
      totalLinear += pda::impl::bicgstab(w, n, rowptr, colidx, linear_tol, linear_max_iters, s, &rel);
      worstRel = std::max(worstRel, rel);
      pda::impl::dot(w, n, w.d.p, w.d.p, pda::impl::RR, s);
      const double dd = pda::impl::read_scalar(w, pda::impl::RR, s);
      if (std::sqrt(dd) < newton_tol) break;  // stop before updating, as Pressio does
      pda::impl::k_axpy<<<pda::impl::g1(n), 256, 0, s>>>(n, -1., w.d.p, d_U);
    }
    totalNewton += it + 1;
    maxNewton = std::max(maxNewton, it + 1);
    t = t + dt;
  }
  PDA_CUDA(cudaStreamSynchronize(s));
  if (info) {
    info[0] = (double)totalNewton;
    info[1] = (double)maxNewton;
    info[2] = (double)totalLinear;
    info[3] = worstRel;
  }
  PDA_API_END
}

}  // extern "C"
